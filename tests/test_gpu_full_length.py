"""GPU solver over the full size and length of every configuration, through the C ABI.

Two checks at every dump step of each configuration's whole run:
  - against the reference: every body's state digest equals the one recorded from the reference built
    with JPH_CROSS_PLATFORM_DETERMINISTIC (tests/golden/full_<name>.npz), i.e. body position, local
    positions and velocities are bit for bit the reference's (NaN payloads aside);
  - against the CPU oracle stepped side by side on all host cores: the same arrays compared exactly,
    NaN masks included, so a failure names the body, the array and the size of the difference.
Configurations: the pinned 30 x 30 cloth (300 steps), the 512-body uneven batch (240 steps; nine large
stiff cloths go non-finite in the reference's own arithmetic and must do so here too), the 64 x 64
differentiable cloth (120 steps), the 256-body differentiable batch (90 steps, forces every step) and
the 256 x 256 cloth on the thread-block-cluster path (600 steps).
"""
import os

import numpy as np
import pytest

from jsb_testlib import Oracle, state_digest
from test_gpu_parity import advance, make_ctx, snapshot
from test_oracle_full import full_scene

pytestmark = pytest.mark.gpu


def compare_exact(got, ref, what):
    for b, (x, y) in enumerate(zip(got, ref)):
        for k, name in enumerate(("position", "local", "velocity")):
            gx, gy = np.asarray(x[k]), np.asarray(y[k])
            nx, ny = np.isnan(gx), np.isnan(gy)
            assert np.array_equal(nx, ny), f"{what}: body {b} {name}: NaN masks differ ({int(nx.sum())} vs {int(ny.sum())})"
            ok = ~nx
            assert np.array_equal(gx[ok], gy[ok]), \
                f"{what}: body {b} {name} differs, max {np.abs(gx[ok].astype(np.float64) - gy[ok]).max()}"


def run_full(jsb, name, with_oracle=True):
    g, scene_bytes, scene = full_scene(name)
    ctx = make_ctx(jsb, scene_bytes, step_forces=True)
    o = Oracle(scene, threads=os.cpu_count() or 1) if with_oracle else None
    cur = 0
    for k, step in enumerate(g["steps"]):
        advance(ctx, int(step) - cur, "graph")
        if o is not None:
            o.step(int(step) - cur)
        cur = int(step)
        try:
            ctx.synchronize()
        except jsb.JsbError as e:  # bodies that blow up in the reference blow up here too
            assert e.status == jsb.JSB_ERR_NONFINITE and g["nan_components"][k].any(), str(e)
        got = [ctx.read_body(b["id"]) for b in ctx.bodies]
        if o is not None:
            compare_exact(got, [o.body(b) for b in range(len(scene.bodies))], f"{name} step {step} vs oracle")
        bad = [b for b, (p, l, v) in enumerate(got) if state_digest(p, l, v) != g["digest"][k, b].tobytes()]
        assert not bad, f"{name} step {step}: {len(bad)} bodies differ from the reference, first {bad[:8]}"
    ctx.close()


@pytest.mark.parametrize("name", ["pinned_cloth", "uneven_batch", "diff_cloth", "diff_batch"])
def test_full_length_vs_reference_and_oracle(jsb, name):
    run_full(jsb, name)


def test_large_cloth_full_length_vs_reference_and_oracle(jsb):
    """The 65,536-vertex cloth over its 600 steps (the oracle runs this one body on one thread)."""
    run_full(jsb, "large_cloth")
