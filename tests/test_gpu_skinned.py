"""Skinned constraints on the GPU through the C ABI (jsb_body_skin_vertices, jsb_body_set_skin_settings)
against the reference's own run (tests/golden/skinned_cloth.npz) and the CPU oracle.

The 16 x 16 cloth skinned to two animated joints (see tests/test_oracle_skinned.py). Bar: body position,
local positions and velocities bitwise equal to the reference at every dumped step and to the oracle at
every step, and the skin block of jsb_body_save_state bitwise equal to the reference's SaveState bytes; on
the whole-step walk (the default), the per-substep walk and the thread-block-cluster path (two cluster
shapes). Differentiable runs do not take skinned bodies and are refused.
"""
import numpy as np
import pytest

from conftest import golden_path
from jsb_testlib import parse_scene
from test_oracle_skinned import MOTION_HEADER, skin_events, skin_from_state

pytestmark = pytest.mark.gpu


PATHS = {"whole_step": (True, None), "per_substep": (False, None), "cluster_2x128": (True, (2, 128)),
         "cluster_4x256": (True, (4, 256))}


@pytest.mark.parametrize("path", list(PATHS))
def test_skinned_cloth_bitwise_vs_reference_and_oracle(jsb, oracle_lib, path):
    step_walk, cluster = PATHS[path]
    g = np.load(golden_path("skinned_cloth"))
    scene_bytes = g["scene"].tobytes()
    scene, _ = parse_scene(scene_bytes)
    nv = int(g["num_vertices"][0])
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    ctx.set_step_walk(step_walk)
    if cluster is not None:
        for mv, t, _ in ctx.bucket_table():
            ctx.set_bucket_config(mv, t, 2)
        ctx.set_cluster_config(*cluster)
    o = oracle_lib(scene)
    ev = skin_events(g)
    dumps = set(int(s) for s in g["steps"])
    for step in range(1, int(g["steps"][-1]) + 1):
        mult, enabled, hard, joints = ev[step]
        ctx.set_skin_settings(0, enabled, mult)
        ctx.skin_vertices(0, joints, hard)
        o.set_skin_settings(0, enabled, mult)
        o.skin_vertices(0, joints, hard)
        ctx.step()
        o.step(1)
        ctx.synchronize()
        pos, loc, vel = ctx.read_body(0)
        opos, oloc, ovel = o.body(0)
        assert np.array_equal(pos, opos) and np.array_equal(loc, oloc) and np.array_equal(vel, ovel), (step, np.abs(loc - oloc).max())
        state = ctx.save_state(0)
        assert len(state) == MOTION_HEADER + 24 * nv + 36 * nv + 48
        assert np.array_equal(skin_from_state(state, nv), o.skin_state(0)), step
        if step in dumps:
            assert np.array_equal(pos, g[f"det_pos_{step}"][0]), step
            assert np.array_equal(loc, g[f"det_local_{step}"]), step
            assert np.array_equal(vel, g[f"det_vel_{step}"]), step
            assert np.array_equal(skin_from_state(state, nv), skin_from_state(g[f"det_state_{step}"].tobytes(), nv)), step
    ctx.close()


def test_skinned_refused_where_unsupported(jsb):
    """Differentiable runs do not take skinned bodies."""
    g = np.load(golden_path("skinned_cloth"))
    ctx = jsb.Context(0)
    ctx.load_scene(g["scene"].tobytes())
    with pytest.raises(jsb.JsbError):
        ctx.adjoint_begin(2, 1)
    ctx.close()
