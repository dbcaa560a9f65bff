"""Two-way coupling on the GPU through the C ABI (jsb_body_set_colliding_shapes), against the reference's
own run (tests/golden/coupling.npz) and the CPU oracle.

Each step every soft body gets the colliding shapes the reference determined for it (a dynamic sphere
and a turned, spinning dynamic box on two trampolines, a turned static box and the floor under a third
cloth), then the batched step runs. Bar: every body's state bitwise equal to the reference
(deterministic build) at every dumped step and to the oracle at every step; the dynamic bodies' velocity
changes read back through jsb_body_shape_velocities give the reference's velocities after each step
bitwise, and the SoftBodyManifold read back through jsb_body_contacts (contact flags, points, normals,
contacted body) is the reference's, bitwise (as in tests/test_oracle_coupling.py); coupling_sensors adds
two sensors, whose contacts read back through jsb_body_sensor_contacts are the manifold's sensor contacts.
The same bar holds with every body forced onto the thread-block-cluster path (mode "cluster").
"""
import numpy as np
import pytest

from conftest import golden_path
from jsb_testlib import parse_scene
from test_oracle_coupling import (check_manifold, check_sensors, check_velocity_changes, manifolds_by_key, register_hulls,
                                  sensors_by_key, tables_by_step)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,mode", [("coupling", "batched"), ("coupling", "plain"), ("coupling_hulls", "batched"),
                                       ("coupling_sensors", "batched"), ("coupling", "cluster"), ("coupling_hulls", "cluster"),
                                       ("coupling_sensors", "cluster")])
def test_coupling_bitwise_vs_reference_and_oracle(jsb, oracle_lib, name, mode):
    g = np.load(golden_path(name))
    scene_bytes = g["scene"].tobytes()
    scene, _ = parse_scene(scene_bytes)
    nv = list(g["num_vertices"])
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    o = oracle_lib(scene)
    gpu_hulls = register_hulls(g, ctx.add_hull)
    assert gpu_hulls == register_hulls(g, o.add_hull)  # (same ids: both count from 0)
    tables = tables_by_step(g, gpu_hulls)
    manifolds = manifolds_by_key(g)
    sensors = sensors_by_key(g)
    ctx.set_contact_readback(True)
    if mode == "cluster":  # every body on the thread-block-cluster path
        for mv, t, _ in ctx.bucket_table():
            ctx.set_bucket_config(mv, t, 2)
        ctx.set_cluster_config(2, 128)
    contacts = sensor_shapes = 0
    dumps = set(int(s) for s in g["steps"])
    changes = 0
    for step in range(1, int(g["steps"][-1]) + 1):
        rows = tables.get(step, [])
        for b in range(len(nv)):
            shapes = [r[2] for r in rows if r[0] == b]
            ctx.set_colliding_shapes(b, shapes)
            o.set_colliding_shapes(b, shapes)
        if mode == "plain":
            ctx.step_plain()
        else:
            ctx.step()
        o.step(1)
        ctx.synchronize()
        out = {b: ctx.shape_velocities(b) for b in range(len(nv))}
        for b in range(len(nv)):
            assert np.array_equal(out[b], o.shape_velocities(b)), (step, b)
        changes += check_velocity_changes(rows, out, g["rigid_after"][step - 1])
        if mode != "plain":
            for b in range(len(nv)):
                c = ctx.contacts(b)
                contacts += check_manifold(manifolds.get((step, b)), b, rows, c["has_contact"], c["points"], c["normals"], c["shape"])
        for b in range(len(nv)):
            mask = ctx.sensor_contacts(b)
            assert mask == o.sensor_contacts(b), (step, b)
            sensor_shapes += check_sensors(sensors.get((step, b)), b, rows, mask)
        off = 0
        for b in range(len(nv)):
            pos, loc, vel = ctx.read_body(b)
            opos, oloc, ovel = o.body(b)
            assert np.array_equal(pos, opos) and np.array_equal(loc, oloc) and np.array_equal(vel, ovel), (step, b)
            if step in dumps:
                assert np.array_equal(pos, g[f"det_pos_{step}"][b]), (step, b)
                assert np.array_equal(loc, g[f"det_local_{step}"][off:off + nv[b]]), (step, b)
                assert np.array_equal(vel, g[f"det_vel_{step}"][off:off + nv[b]]), (step, b)
            off += nv[b]
    ctx.close()
    assert changes > 50, changes
    assert mode == "plain" or contacts > 1000, contacts
    assert name != "coupling_sensors" or (len(sensors) > 100 and sensor_shapes > len(sensors)), (len(sensors), sensor_shapes)


def test_coupling_refused_where_unsupported(jsb):
    """Graph replays and differentiable runs do not take host-determined shapes."""
    g = np.load(golden_path("coupling"))
    tables = tables_by_step(g)
    rows = tables[20]
    ctx = jsb.Context(0)
    ctx.load_scene(g["scene"].tobytes())
    ctx.set_colliding_shapes(0, [r[2] for r in rows if r[0] == 0])
    with pytest.raises(jsb.JsbError):
        ctx.step_graph(2, 1)
    with pytest.raises(jsb.JsbError):
        ctx.adjoint_begin(2, 1)
    ctx.set_colliding_shapes(0, None)
    ctx.step_graph(2, 1)
    ctx.close()
