"""Generates the golden fixtures in tests/golden/ by running the reference itself.

Requires oracle/_ref (built from the reference sources with oracle/Makefile.ref, where the reference
is available):

    make -f oracle/Makefile.ref REF=<path to JoltPhysics> -j8
    python tests/golden/make_golden.py

For each case the reference driver (oracle/ref_driver.cpp) builds the seeded scene with Jolt's own
SoftBodySharedSettings::CreateConstraints/Optimize, steps it with PhysicsSystem::Update, and dumps
world positions. A fixture stores the serialised scene (settings bytes written by Jolt) and, per dump
step, each body's position, local vertex positions and velocities, from the deterministic build
(JPH_CROSS_PLATFORM_DETERMINISTIC) and, for the final step, from the default FMA build.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from jsb_testlib import parse_dump, run_reference  # noqa: E402

CASES = {
    # name: (scene, params, dump steps)
    "pinned_cloth": ("pinned_cloth", {}, [1, 10, 100, 300]),
    "uneven_small": ("uneven_batch", dict(n_cloth=6, n_cube=3, cloth_max=20, cube_max=5, steps=40), [1, 20, 40]),
    "large_cloth_32": ("large_cloth", dict(n=32, steps=120), [1, 60, 120]),
    "diff_cloth_16": ("diff_cloth", dict(n=16, steps=40), [1, 40]),
    "diff_batch_small": ("diff_batch", dict(n_cloth=4, n_cube=2, steps=30), [1, 30]),
}


def make(name: str, scene: str, params: dict, steps: list[int]):
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for variant in ("det", "fast"):
            path = os.path.join(tmp, f"{variant}.bin")
            run_reference(variant, scene, path, dump=",".join(str(s) for s in [0] + steps), **params)
            sc, dumps = parse_dump(path)
            if variant == "det":
                out["scene"] = np.frombuffer(sc.raw, np.uint8)
                out["steps"] = np.array(steps, np.int32)
                out["num_vertices"] = np.array([b.num_vertices for b in sc.bodies], np.int64)
            for d in dumps[1:]:
                if variant == "fast" and d.step != steps[-1]:
                    continue
                out[f"{variant}_pos_{d.step}"] = np.stack(d.positions).astype(np.float32)
                out[f"{variant}_local_{d.step}"] = np.concatenate(d.local).astype(np.float32)
                out[f"{variant}_vel_{d.step}"] = np.concatenate(d.velocities).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


if __name__ == "__main__":
    for name, (scene, params, steps) in CASES.items():
        make(name, scene, params, steps)
        print("wrote", name)
