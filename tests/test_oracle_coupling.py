"""The CPU oracle's host-determined colliding shapes against the reference's two-way coupling run
(tests/golden/coupling.npz, written by tests/golden/make_golden.py from the reference driver).

Three cloths under a static floor: a dynamic sphere and a turned, spinning dynamic box fall onto two
trampolines, a third cloth onto a static turned box (coupling_hulls adds a fourth cloth falling onto a
static convex hull, with a small dynamic hull dropped onto it; coupling_sensors adds a static box sensor under the
first trampoline and a kinematic sphere sensor rising through the second cloth). Jolt's own rigid-body solver moves the rigid bodies;
each step every soft body's colliding shapes are fed to the oracle as the reference determined them
(transforms, combined friction / restitution, the dynamic bodies' mass, inertia and velocities). Bar:
- every soft body's state bitwise equal to the reference (deterministic build) at every dumped step;
- the dynamic bodies' velocity changes (UpdateRigidBodyVelocities, SoftBodyMotionProperties.cpp:923-935):
  the rigid body's velocity when collected plus the oracle's change equals the reference's velocity after
  the step, bitwise;
- every step's SoftBodyManifold (what OnSoftBodyContactAdded sees): contact flags, local contact points and
  normals bitwise, and the contacted rigid body;
- its sensor contacts (GetSensorContactBodyID): the sensors a vertex penetrated (DetermineSensorCollisions,
  SoftBodyMotionProperties.cpp:267-289).
"""
import struct

import numpy as np
import pytest

from conftest import golden_path
from jsb_testlib import SHAPE_FMT, parse_scene


def tables_by_step(g, hull_ids=None):
    """Per step: (soft body, rigid body, jsb_colliding_shape bytes, the rigid body's velocities when collected).
    hull_ids: rigid index -> id of its registered hull, written into the hulls' records."""
    out = {}
    for k in range(len(g["tables_step"])):
        shape = g["tables_shape"][k].tobytes()
        rigid = int(g["tables_rigid"][k])
        if hull_ids is not None and struct.unpack_from("<i", shape, 0)[0] == 4:
            shape = shape[:-4] + struct.pack("<I", hull_ids[rigid])
        out.setdefault(int(g["tables_step"][k]), []).append((int(g["tables_body"][k]), rigid, shape, g["tables_rigid_velocity"][k]))
    return out


def register_hulls(g, add) -> dict:
    """Registers the golden's convex hulls with add(points, planes, faces); returns rigid index -> id."""
    ids = {}
    for key in sorted(k for k in g.files if k.endswith("_points") and k.startswith("hull")):
        r = int(key[4:-7])
        counts, idx = g[f"hull{r}_counts"], g[f"hull{r}_indices"]
        faces, off = [], 0
        for c in counts:
            faces.append(idx[off:off + c])
            off += c
        ids[r] = add(g[key], g[f"hull{r}_planes"], faces)
    return ids


def world_delta(local_new, local_old):
    """inContext.mCenterOfMassTransform.Multiply3x3(new - old) with the soft body's identity rotation, in
    float32 with Mat44::Multiply3x3's order: (c0 x + c1 y) + c2 z."""
    d = (np.asarray(local_new, np.float32) - np.asarray(local_old, np.float32)).astype(np.float32)
    one, zero = np.float32(1), np.float32(0)
    cols = [(one, zero, zero), (zero, one, zero), (zero, zero, one)]
    return np.array([(cols[0][i] * d[0] + cols[1][i] * d[1]) + cols[2][i] * d[2] for i in range(3)], np.float32)


def check_velocity_changes(rows, shape_out_by_body, after):
    """rows: the step's (body, rigid, shape bytes, world velocities when collected); shape_out_by_body:
    per body the solver's (updated, lin[3], ang[3]) per shape; after: the reference's (num_rigid, 6)."""
    per_body_index = {}
    checked = 0
    for body, rigid, shape, vel0 in rows:
        k = per_body_index.get(body, 0)
        per_body_index[body] = k + 1
        v = struct.unpack(SHAPE_FMT, shape)
        if v[1] != 2:
            continue
        out = shape_out_by_body[body][k]
        lin_in, ang_in = np.array(v[37:40], np.float32), np.array(v[40:43], np.float32)
        if out[0] == 0:
            assert np.array_equal(out[1:4], lin_in) and np.array_equal(out[4:7], ang_in)
            assert np.array_equal(after[rigid], vel0), (body, rigid)
            continue
        lin = (vel0[:3] + world_delta(out[1:4], lin_in)).astype(np.float32)
        ang = (vel0[3:] + world_delta(out[4:7], ang_in)).astype(np.float32)
        assert np.array_equal(lin, after[rigid][:3]), (body, rigid, lin, after[rigid][:3])
        assert np.array_equal(ang, after[rigid][3:]), (body, rigid, ang, after[rigid][3:])
        checked += 1
    return checked


def manifolds_by_key(g):
    """(step, soft body) -> the reference's SoftBodyManifold: (has (N,), points (N, 3), normals (N, 3), rigid (N,))."""
    out, off = {}, 0
    nv = list(g["num_vertices"])
    for st, b in zip(g["manifold_step"], g["manifold_body"]):
        n = nv[int(b)]
        out[(int(st), int(b))] = (g["manifold_has"][off:off + n], g["manifold_point"][off:off + n], g["manifold_normal"][off:off + n],
                                  g["manifold_rigid"][off:off + n])
        off += n
    return out


def sensors_by_key(g):
    """(step, soft body) -> the rigid indices of the reference manifold's sensor contacts."""
    out = {}
    if "sensor_step" in g.files:
        for st, b, r in zip(g["sensor_step"], g["sensor_body"], g["sensor_rigid"]):
            out.setdefault((int(st), int(b)), set()).add(int(r))
    return out


def check_sensors(ref, body, rows, mask):
    """A solver's sensor mask of one body and step (bit k: table shape k) against the reference's sensor
    contacts (a set of rigid indices). Returns the number of sensor shapes of the body in the step."""
    rigid_of_shape = [r[1] for r in rows if r[0] == body]
    got = {rigid_of_shape[k] for k in range(len(rigid_of_shape)) if (mask >> k) & 1}
    assert got == (ref or set()), (body, got, ref)
    return sum(1 for r in rows if r[0] == body and struct.unpack_from("<i", r[2], 4)[0] == 3)


def check_manifold(ref, body, rows, has, points, normals, shapes):
    """A solver's manifold of one body and step (has, points, normals, shape index per vertex) against the
    reference's (None: OnSoftBodyContactAdded was not called, so no vertex may touch)."""
    has = np.asarray(has).astype(bool)
    if ref is None:
        assert not has.any()
        return 0
    rhas, rpts, rnrm, rrig = ref
    assert np.array_equal(has, rhas.astype(bool))
    assert np.array_equal(np.asarray(points)[has], rpts[has])
    assert np.array_equal(np.asarray(normals)[has], rnrm[has])
    rigid_of_shape = [r[1] for r in rows if r[0] == body]
    assert [rigid_of_shape[s] for s in np.asarray(shapes)[has]] == list(rrig[has])
    return int(has.sum())


@pytest.mark.parametrize("name", ["coupling", "coupling_hulls", "coupling_sensors"])
def test_oracle_coupling_bitwise_vs_reference(oracle_lib, name):
    g = np.load(golden_path(name))
    scene, _ = parse_scene(g["scene"].tobytes())
    nv = list(g["num_vertices"])
    o = oracle_lib(scene)
    o.set_contact_readback(True)
    tables = tables_by_step(g, register_hulls(g, o.add_hull))
    manifolds = manifolds_by_key(g)
    sensors = sensors_by_key(g)
    dumps = set(int(s) for s in g["steps"])
    changes = contacts = sensor_shapes = 0
    for step in range(1, int(g["steps"][-1]) + 1):
        rows = tables.get(step, [])
        for b in range(len(nv)):
            o.set_colliding_shapes(b, [r[2] for r in rows if r[0] == b])
        o.step(1)
        changes += check_velocity_changes(rows, {b: o.shape_velocities(b) for b in range(len(nv))}, g["rigid_after"][step - 1])
        for b in range(len(nv)):
            m = o.contacts(b)
            contacts += check_manifold(manifolds.get((step, b)), b, rows, m[:, 0], m[:, 1:4], m[:, 4:7], m[:, 7].astype(np.int64))
            sensor_shapes += check_sensors(sensors.get((step, b)), b, rows, o.sensor_contacts(b))
        if step in dumps:
            off = 0
            for b in range(len(nv)):
                pos, loc, vel = o.body(b)
                assert np.array_equal(pos, g[f"det_pos_{step}"][b]), (step, b)
                assert np.array_equal(loc, g[f"det_local_{step}"][off:off + nv[b]]), (step, b)
                assert np.array_equal(vel, g[f"det_vel_{step}"][off:off + nv[b]]), (step, b)
                off += nv[b]
    assert changes > 50, changes  # the sphere and the box are pushed by their trampolines most of the run
    assert contacts > 1000, contacts
    if name == "coupling_sensors":
        assert len(sensors) > 100 and sensor_shapes > len(sensors), (len(sensors), sensor_shapes)
