"""The CPU oracle against the reference over the full size and length of every configuration.

Fixtures tests/golden/full_<name>.npz (written by tests/golden/make_golden.py from the reference built
with JPH_CROSS_PLATFORM_DETERMINISTIC) hold, per dump step and body, a digest of the body's state
(jsb_testlib.state_digest), the number of NaN position components, and the SHA-256 of the scene bytes
Jolt's own CreateConstraints / Optimize / SaveBinaryState wrote. Bar:
  - the scene library's settings mirror writes exactly those scene bytes at full size;
  - the float oracle reproduces every body's state bit for bit at every dump step (NaN payloads aside,
    which the digest canonicalises), including the bodies that go non-finite in the reference itself.
The 256 x 256 cloth (one body, 600 steps) runs on one thread and takes about a minute.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import golden_path
from jsb_testlib import Oracle, parse_scene, state_digest
from scenes import build_scene

FULL = ["pinned_cloth", "uneven_batch", "diff_cloth", "diff_batch", "large_cloth"]


def load_full(name):
    import json

    g = np.load(golden_path(f"full_{name}"))
    params = json.loads(g["params"].tobytes().decode())
    scene_name = params.pop("scene")
    return g, scene_name, params


def full_scene(name):
    """(fixture, scene bytes built by the scene library, parsed scene); checks the bytes against Jolt's."""
    g, scene_name, params = load_full(name)
    scene_bytes = build_scene(scene_name, **params)
    assert hashlib.sha256(scene_bytes).digest() == g["scene_sha256"].tobytes(), \
        f"{name}: the settings mirror's scene bytes differ from Jolt's"
    scene, _ = parse_scene(scene_bytes)
    return g, scene_bytes, scene


def digest_mismatches(g, k, states):
    """Bodies whose state digest differs from the fixture's at dump index k (states: (pos, local, vel) per body)."""
    bad = []
    for b, (pos, loc, vel) in enumerate(states):
        if state_digest(pos, loc, vel) != g["digest"][k, b].tobytes():
            bad.append(b)
    return bad


@pytest.mark.parametrize("name", FULL)
def test_oracle_full_length_vs_reference(name, oracle_lib):
    g, _, scene = full_scene(name)
    o = Oracle(scene, threads=os.cpu_count() or 1)
    cur = 0
    for k, step in enumerate(g["steps"]):
        o.step(int(step) - cur)
        cur = int(step)
        states = [o.body(b) for b in range(len(scene.bodies))]
        bad = digest_mismatches(g, k, states)
        assert not bad, f"{name} step {step}: {len(bad)} bodies differ from the reference, first {bad[:8]}"
        nans = [int(np.isnan(s[1]).sum()) for s in states]
        assert nans == list(g["nan_components"][k]), f"{name} step {step}: NaN pattern differs"


def test_diff_cloth_gradient_conditioning(oracle_lib):
    """Why the differentiable cloth's gradients are checked against finite differences only over a short
    horizon: FP64 central differences (the oracle in double precision) of its MSE loss, on 8 edge
    compliances and 8 initial velocities, move by more than 1e-2 relative when the initial positions move
    by 1e-7 m and the loss is taken at steps 60 and 120 (the stated configuration), and by less than 1e-3
    (but not much less) when it is taken at steps 3 and 6. No FP32 trajectory can match a gradient that
    is not stable under perturbations far below its own rounding, so the full-length gradient is checked
    along the GPU's own trajectory instead (tests/test_gpu_gradients_full.py)."""
    from jsb_testlib import blob_arrays, blob_compliance, run64

    scene, _ = parse_scene(build_scene("diff_cloth"))
    x0, v0, _ = blob_arrays(scene.bodies[0].blob)
    ec, _ = blob_compliance(scene.bodies[0].blob)
    rng = np.random.default_rng(1)
    ec_t = ec * np.exp(0.3 * rng.standard_normal(ec.shape))
    pe = rng.choice(len(ec), 8, replace=False)
    pv = [(int(rng.integers(len(v0))), int(rng.integers(3))) for _ in range(8)]
    x0p = x0 + 1e-7 * rng.standard_normal(x0.shape)

    def sensitivity(steps):
        tgt = run64(scene, 0, max(steps), set(steps), edge=ec_t)

        def loss(x, e, v):
            out = run64(scene, 0, max(steps), set(steps), x0=x, edge=e, v0=v)
            return sum(float(((out[s] - tgt[s]) ** 2).sum()) for s in steps)

        def grad(x):
            g = []
            for i in pe:
                a, b = ec.copy(), ec.copy()
                a[i] *= 1 + 1e-6
                b[i] *= 1 - 1e-6
                g.append((loss(x, a, v0) - loss(x, b, v0)) / (2e-6 * ec[i]))
            for idx in pv:
                a, b = v0.copy(), v0.copy()
                a[idx] += 1e-6
                b[idx] -= 1e-6
                g.append((loss(x, ec, a) - loss(x, ec, b)) / 2e-6)
            return np.array(g)

        g0, g1 = grad(x0), grad(x0p)
        return max(np.linalg.norm(g1[:8] - g0[:8]) / np.linalg.norm(g0[:8]), np.linalg.norm(g1[8:] - g0[8:]) / np.linalg.norm(g0[8:]))

    long_run, short_run = sensitivity((60, 120)), sensitivity((3, 6))
    print(f"relative change of the FP64 FD gradient under a 1e-7 m perturbation: steps 60/120 {long_run:.3e}, "
          f"steps 3/6 {short_run:.3e}")
    assert long_run > 1e-2 and short_run < 1e-3
