"""Skinned constraints in the CPU oracle against the reference's own run (tests/golden/skinned_cloth.npz,
written by tests/golden/make_golden.py from the reference driver).

A 16 x 16 cloth skinned to two animated joints: SoftBodyMotionProperties::SkinVertices before every step
(hard skinning on the first), the maximum distance multiplier raised to 1.5 from step 40 and skin
constraints switched off for steps 61-65. Bar: every dumped step's body position, local positions and
velocities bitwise, and the skin states (previous skinned position, skinned position, normal) bitwise
against the reference's SaveState bytes.
"""
import numpy as np

from conftest import golden_path
from jsb_testlib import parse_scene

MOTION_HEADER = 101  # MotionProperties::SaveState bytes before the vertices


def skin_from_state(state: bytes, nv: int) -> np.ndarray:
    """The SkinState block of SoftBodyMotionProperties::SaveState bytes: (N, 3, 3)."""
    off = MOTION_HEADER + 24 * nv
    return np.frombuffer(state, np.float32, 9 * nv, off).reshape(nv, 3, 3)


def skin_events(g):
    """step -> (multiplier, enabled, hard, joints (2, 16))."""
    return {int(s): (float(m), bool(e), bool(h), j) for s, m, e, h, j in
            zip(g["skin_step"], g["skin_mult"], g["skin_enabled"], g["skin_hard"], g["skin_joints"])}


def test_oracle_skinned_cloth_bitwise_vs_reference(oracle_lib):
    g = np.load(golden_path("skinned_cloth"))
    scene, _ = parse_scene(g["scene"].tobytes())
    nv = int(g["num_vertices"][0])
    o = oracle_lib(scene)
    ev = skin_events(g)
    dumps = set(int(s) for s in g["steps"])
    for step in range(1, int(g["steps"][-1]) + 1):
        mult, enabled, hard, joints = ev[step]
        o.set_skin_settings(0, enabled, mult)
        o.skin_vertices(0, joints, hard)
        o.step(1)
        if step in dumps:
            pos, loc, vel = o.body(0)
            assert np.array_equal(pos, g[f"det_pos_{step}"][0]), step
            assert np.array_equal(loc, g[f"det_local_{step}"]), (step, np.abs(loc - g[f"det_local_{step}"]).max())
            assert np.array_equal(vel, g[f"det_vel_{step}"]), step
            assert np.array_equal(o.skin_state(0), skin_from_state(g[f"det_state_{step}"].tobytes(), nv)), step
