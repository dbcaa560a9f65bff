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
