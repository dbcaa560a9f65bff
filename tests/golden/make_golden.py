"""Generates the golden fixtures in tests/golden/ by running the reference itself.

Requires oracle/_ref (built from the reference sources with oracle/Makefile.ref, where the reference
is available):

    make -f oracle/Makefile.ref REF=<path to JoltPhysics> -j8
    python tests/golden/make_golden.py

For each case the reference driver (oracle/ref_driver.cpp) builds the seeded scene with Jolt's own
SoftBodySharedSettings::CreateConstraints/Optimize, steps it with PhysicsSystem::Update, and dumps
world positions. A fixture stores the serialised scene (settings bytes written by Jolt) and, per dump
step, each body's position, local vertex positions and velocities, from the deterministic build
(JPH_CROSS_PLATFORM_DETERMINISTIC) and, for the final step (every step for the pinned cloth), from the
default FMA build.

The full-size configurations (FULL_CASES) run over their whole stated length; their states are too
large to commit, so those fixtures ("full_<name>.npz") keep per dump step and body a 16-byte digest of
the deterministic build's state (jsb_testlib.state_digest: body position, local positions and
velocities, NaNs canonicalised), the count of NaN position components, and the largest world-position
difference between the two builds (finite vertices only), plus the SHA-256 of the scene bytes Jolt
wrote, against which the scene library's mirror output is checked.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from jsb_testlib import parse_dump, run_reference, state_digest  # noqa: E402

CASES = {
    # name: (scene, params, dump steps)
    "pinned_cloth": ("pinned_cloth", {}, [1, 10, 100, 300]),
    "uneven_small": ("uneven_batch", dict(n_cloth=6, n_cube=3, cloth_max=20, cube_max=5, steps=40), [1, 20, 40]),
    "large_cloth_32": ("large_cloth", dict(n=32, steps=120), [1, 60, 120]),
    "diff_cloth_16": ("diff_cloth", dict(n=16, steps=40), [1, 40]),
    "diff_batch_small": ("diff_batch", dict(n_cloth=4, n_cube=2, steps=30), [1, 30]),
    # sleeping allowed: bodies that come to rest on the floor fall asleep and stop being stepped
    # every static shape type: capsule, cylinders, sphere, box floor
    "shapes_drop": ("shapes_drop", {}, [1, 40, 80, 150]),
    "sleep_small": ("uneven_batch", dict(n_cloth=6, n_cube=3, cloth_max=20, cube_max=5, steps=200, sleep=1), [1, 60, 120, 160, 200]),
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
                if variant == "fast" and d.step != steps[-1] and name != "pinned_cloth":
                    continue  # (the pinned cloth keeps the default build at every step: its stated tolerance)
                if variant == "det":  # MotionProperties::mSleepTestTimer from the SaveState bytes (offset 96)
                    out[f"det_timer_{d.step}"] = np.array([np.frombuffer(st, np.float32, 1, 96)[0] for st in d.states], np.float32)
                out[f"{variant}_pos_{d.step}"] = np.stack(d.positions).astype(np.float32)
                out[f"{variant}_local_{d.step}"] = np.concatenate(d.local).astype(np.float32)
                out[f"{variant}_vel_{d.step}"] = np.concatenate(d.velocities).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def make_coupling(name: str = "coupling", steps: int = 90, dump: tuple = (1, 10, 17, 18, 19, 20, 30, 45, 60, 75, 90), **params):
    """Two-way coupling (rigid bodies simulated by the reference's own solver; params: scene parameters,
    hulls=1 adds convex hulls, sensors=1 sensors): per dump step the
    deterministic build's soft-body states, and for every step each soft body's colliding shapes as the
    reference determined them (tables_*: jsb_colliding_shape bytes, soft body, rigid body, the rigid body's
    world velocities when collected) and the rigid bodies' velocities after the step."""
    from jsb_testlib import SHAPE_BYTES, parse_tables

    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        path, tab = os.path.join(tmp, "det.bin"), os.path.join(tmp, "det.tab")
        run_reference("det", "coupling", path, dump=",".join(str(s) for s in [0, *dump]), steps=steps, tables=tab, **params)
        sc, dumps = parse_dump(path)
        t = parse_tables(tab, len(sc.bodies))
    out["scene"] = np.frombuffer(sc.raw, np.uint8)
    out["steps"] = np.array(dump, np.int32)
    out["num_vertices"] = np.array([b.num_vertices for b in sc.bodies], np.int64)
    for d in dumps[1:]:
        out[f"det_pos_{d.step}"] = np.stack(d.positions).astype(np.float32)
        out[f"det_local_{d.step}"] = np.concatenate(d.local).astype(np.float32)
        out[f"det_vel_{d.step}"] = np.concatenate(d.velocities).astype(np.float32)
    rows = [(st, *r) for st in sorted(t["steps"]) for r in t["steps"][st]]
    out["tables_step"] = np.array([r[0] for r in rows], np.int32)
    out["tables_body"] = np.array([r[1] for r in rows], np.int32)
    out["tables_rigid"] = np.array([r[2] for r in rows], np.int32)
    out["tables_shape"] = np.frombuffer(b"".join(r[3] for r in rows), np.uint8).reshape(len(rows), SHAPE_BYTES)
    out["tables_rigid_velocity"] = np.stack([r[4] for r in rows]).astype(np.float32)
    out["rigid_after"] = t["rigid_after"]
    keys = sorted(t["manifolds"])  # the manifolds OnSoftBodyContactAdded saw: (step, body) -> per vertex
    out["manifold_step"] = np.array([k[0] for k in keys], np.int32)
    out["manifold_body"] = np.array([k[1] for k in keys], np.int32)
    if keys:
        out["manifold_has"] = np.concatenate([t["manifolds"][k]["has"] for k in keys]).astype(np.uint8)
        out["manifold_point"] = np.concatenate([t["manifolds"][k]["point"] for k in keys]).astype(np.float32)
        out["manifold_normal"] = np.concatenate([t["manifolds"][k]["normal"] for k in keys]).astype(np.float32)
        out["manifold_rigid"] = np.concatenate([t["manifolds"][k]["rigid"] for k in keys]).astype(np.int32)
    sens = [(k[0], k[1], r) for k in sorted(t["sensors"]) for r in t["sensors"][k]]  # manifold sensor contacts
    out["sensor_step"] = np.array([x[0] for x in sens], np.int32)
    out["sensor_body"] = np.array([x[1] for x in sens], np.int32)
    out["sensor_rigid"] = np.array([x[2] for x in sens], np.int32)
    for r, (pts, planes, faces) in t["hulls"].items():  # convex hulls as ConvexHullShape holds them
        out[f"hull{r}_points"] = pts
        out[f"hull{r}_planes"] = planes
        out[f"hull{r}_counts"] = np.array([len(f) for f in faces], np.uint32)
        out[f"hull{r}_indices"] = np.concatenate([np.asarray(f, np.uint32) for f in faces])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


# name: (scene, params, dump steps): every BASELINE configuration at its full size and length
FULL_CASES = {
    "pinned_cloth": ("pinned_cloth", {}, [1, 100, 200, 300]),
    "uneven_batch": ("uneven_batch", {}, [1, 60, 120, 180, 240]),
    "large_cloth": ("large_cloth", {}, [1, 100, 300, 600]),
    "diff_cloth": ("diff_cloth", {}, [1, 60, 120]),
    "diff_batch": ("diff_batch", {}, [1, 45, 90]),
}


def make_skinned(name: str = "skinned_cloth", steps: int = 90, dump: tuple = (1, 2, 10, 39, 40, 60, 62, 66, 90)):
    """A skinned cloth (skinned constraints, SkinVertices before every step): per dump step the
    deterministic build's states (with the SaveState bytes, skin states included), and per step the
    joint matrices relative to the body's centre of mass, the max-distance multiplier, the skin switch and
    the hard-skinning flag the driver passed."""
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        path, sk = os.path.join(tmp, "det.bin"), os.path.join(tmp, "det.skin")
        run_reference("det", "skinned_cloth", path, dump=",".join(str(s) for s in [0, *dump]), steps=steps, skin=sk)
        sc, dumps = parse_dump(path)
        buf = open(sk, "rb").read()
    assert buf[:4] == b"JSBK"
    rec = np.dtype([("step", "<i4"), ("body", "<u4"), ("mult", "<f4"), ("enabled", "<u4"), ("hard", "<u4"), ("joints", "<f4", (2, 16))])
    ev = np.frombuffer(buf, rec, (len(buf) - 4) // rec.itemsize, 4)
    out["scene"] = np.frombuffer(sc.raw, np.uint8)
    out["steps"] = np.array(dump, np.int32)
    out["num_vertices"] = np.array([b.num_vertices for b in sc.bodies], np.int64)
    for d in dumps[1:]:
        out[f"det_pos_{d.step}"] = np.stack(d.positions).astype(np.float32)
        out[f"det_local_{d.step}"] = np.concatenate(d.local).astype(np.float32)
        out[f"det_vel_{d.step}"] = np.concatenate(d.velocities).astype(np.float32)
        out[f"det_state_{d.step}"] = np.frombuffer(d.states[0], np.uint8)
    for k in ("step", "body", "mult", "enabled", "hard", "joints"):
        out[f"skin_{k}"] = ev[k].copy()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def make_full(name: str, scene: str, params: dict, steps: list[int], threads: int):
    import hashlib
    import json

    out = {"params": np.frombuffer(json.dumps({"scene": scene, **params}).encode(), np.uint8), "steps": np.array(steps, np.int32)}
    with tempfile.TemporaryDirectory() as tmp:
        dumps_by = {}
        for variant in ("det", "fast"):
            path = os.path.join(tmp, f"{variant}.bin")
            run_reference(variant, scene, path, dump=",".join(str(s) for s in steps), threads=threads, **params)
            sc, dumps = parse_dump(path)
            if variant == "det":
                out["scene_sha256"] = np.frombuffer(hashlib.sha256(sc.raw).digest(), np.uint8)
                out["num_vertices"] = np.array([b.num_vertices for b in sc.bodies], np.int64)
            dumps_by[variant] = dumps
            os.remove(path)
    det, fast = dumps_by["det"], dumps_by["fast"]
    nb = len(out["num_vertices"])
    digest = np.zeros((len(steps), nb, 16), np.uint8)
    nans = np.zeros((len(steps), nb), np.int32)
    fast_dev = np.zeros((len(steps), nb), np.float64)
    for k, (d, f) in enumerate(zip(det, fast)):
        assert d.step == steps[k] and f.step == steps[k]
        for b in range(nb):
            digest[k, b] = np.frombuffer(state_digest(d.positions[b], d.local[b], d.velocities[b]), np.uint8)
            nans[k, b] = int(np.isnan(d.local[b]).sum())
            wd, wf = d.world(b), f.world(b)
            ok = np.isfinite(wd).all(axis=1) & np.isfinite(wf).all(axis=1)
            fast_dev[k, b] = float(np.abs(wd[ok] - wf[ok]).max()) if ok.any() else 0.0
    out.update(digest=digest, nan_components=nans, fast_max_dev=fast_dev)
    np.savez_compressed(os.path.join(HERE, f"full_{name}.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1:]
    for name, (scene, params, steps) in CASES.items():
        if not which or name in which:
            make(name, scene, params, steps)
            print("wrote", name)
    if not which or "coupling" in which:
        make_coupling()
        print("wrote coupling")
    if not which or "coupling_hulls" in which:  # + a static and a dynamic convex hull under a fourth cloth
        make_coupling("coupling_hulls", hulls=1)
        print("wrote coupling_hulls")
    if not which or "skinned_cloth" in which:  # skinned constraints driven by two animated joints
        make_skinned()
        print("wrote skinned_cloth")
    if not which or "coupling_sensors" in which:  # + a static box sensor and a rising kinematic sphere sensor
        make_coupling("coupling_sensors", sensors=1)
        print("wrote coupling_sensors")
    for name, (scene, params, steps) in FULL_CASES.items():
        if not which or f"full_{name}" in which:
            make_full(name, scene, params, steps, threads=os.cpu_count() or 1)
            print("wrote", f"full_{name}")
