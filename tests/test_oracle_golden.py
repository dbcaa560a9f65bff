"""The CPU oracle against the reference's own outputs (golden fixtures made by tests/golden/make_golden.py).

The float oracle must reproduce the reference built with JPH_CROSS_PLATFORM_DETERMINISTIC bit for bit;
against the default (FMA) build the stated tolerance is max vertex error <= 1e-5 m after 1 step and
<= 1e-3 m at the last dumped step.
"""
import numpy as np
import pytest

from conftest import golden_path
from jsb_testlib import parse_scene

CASES = ["pinned_cloth", "uneven_small", "large_cloth_32", "diff_cloth_16", "diff_batch_small", "sleep_small", "shapes_drop"]


def load(name):
    g = np.load(golden_path(name))
    scene, _ = parse_scene(g["scene"].tobytes())
    return g, scene


def split(arr, nv):
    out, off = [], 0
    for n in nv:
        out.append(arr[off:off + n])
        off += n
    return out


@pytest.mark.parametrize("name", CASES)
def test_oracle_bitwise_vs_reference(name, oracle_lib):
    g, scene = load(name)
    nv = list(g["num_vertices"])
    o = oracle_lib(scene)
    cur = 0
    for step in g["steps"]:
        o.step(int(step) - cur)
        cur = int(step)
        ref_pos = g[f"det_pos_{step}"]
        ref_loc = split(g[f"det_local_{step}"], nv)
        ref_vel = split(g[f"det_vel_{step}"], nv)
        for b in range(len(nv)):
            pos, loc, vel = o.body(b)
            assert np.array_equal(pos, ref_pos[b]), (name, step, b)
            assert np.array_equal(loc, ref_loc[b]), (name, step, b)
            assert np.array_equal(vel, ref_vel[b]), (name, step, b)
            if f"det_timer_{step}" in g:  # sleep timers (MotionProperties::mSleepTestTimer)
                assert np.float32(o.sleep_timer(b)) == g[f"det_timer_{step}"][b], (name, step, b)


@pytest.mark.parametrize("name", ["pinned_cloth"])
def test_oracle_within_tolerance_of_fma_build(name, oracle_lib):
    """The stated bar (pinned cloth, 300 steps): <= 1e-3 m from the reference's default FMA build.

    (On the colliding batch scenes the two reference builds themselves drift apart by a few mm, so the
    bar is only meaningful where it was stated.)"""
    g, scene = load(name)
    nv = list(g["num_vertices"])
    last = int(g["steps"][-1])
    o = oracle_lib(scene)
    o.step(last)
    ref_pos = g[f"fast_pos_{last}"].astype(np.float64)
    ref_loc = split(g[f"fast_local_{last}"].astype(np.float64), nv)
    err = 0.0
    for b in range(len(nv)):
        pos, loc, _ = o.body(b)
        err = max(err, np.abs((loc.astype(np.float64) + pos) - (ref_loc[b] + ref_pos[b])).max())
    assert err <= 1e-3, err


def test_fp64_reevaluation_close(oracle_lib):
    """FP64 evaluation of the same constraint order stays near the FP32 result for the pinned cloth.

    The FP32 reference quantises the dihedral angle of near-flat triangle pairs (sqrt(1 - |d|) with
    |d| close to 1 resolves steps of about 2.4e-4 rad), so the FP32/FP64 gap is ~1e-4 m after one step
    and stays at the mm level; it is reported, not a parity bar."""
    g, scene = load("pinned_cloth")
    o32 = oracle_lib(scene)
    o64 = oracle_lib(scene, use_double=True)
    o32.step(1)
    o64.step(1)
    e1 = np.abs(o32.world_f64(0) - o64.world_f64(0)).max()
    o32.step(299)
    o64.step(299)
    e300 = np.abs(o32.world_f64(0) - o64.world_f64(0)).max()
    assert e1 <= 1e-3 and e300 <= 1e-2, (e1, e300)
