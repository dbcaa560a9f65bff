"""The allocation-free single-body step (jsb_step_body_noalloc) against the regular context step.

jsb_step_body_noalloc exists for callers that cannot call cudaMalloc (engines that hand out all device
memory from their own arenas, frame loops that must not stall on an allocation): its scratch is a static
device array inside the library and the caller passes the body's state in its own device memory. Here the
caller's memory comes from torch; the entry point itself allocates nothing. Two calls in a row must give
bit-identical results to two jsb_step calls of a one-body context (the tolerance of all GPU parity tests).
This file is collected last so that a failure here cannot hide the other GPU tests.
"""
import ctypes
import struct

import numpy as np
import pytest

from conftest import golden_path
from jsb_testlib import COLLIDER_FMT, parse_scene
from scenes import build_scene

pytestmark = pytest.mark.gpu


def body_arrays(blob):
    n = struct.unpack_from("<I", blob, 0)[0]
    v = np.frombuffer(blob, np.float32, 7 * n, 4).reshape(n, 7)
    x = np.concatenate([v[:, 0:3], v[:, 6:7]], axis=1).astype(np.float32)
    vel = np.concatenate([v[:, 3:6], np.zeros((n, 1), np.float32)], axis=1)
    return x, vel


def initial_state(x, position):
    """jsb_body_state after SoftBodyMotionProperties::Initialize: bounds = predicted bounds."""
    bmin, bmax = x[:, :3].min(axis=0), x[:, :3].max(axis=0)
    return np.concatenate([np.asarray(position, np.float32), bmin, bmax, bmin, bmax, np.zeros(6, np.float32)]).astype(np.float32)


def run_noalloc(jsb, scene, body, steps):
    import torch

    b = scene.bodies[body]
    x, vel = body_arrays(b.blob)
    xd = torch.from_numpy(x).cuda()
    vd = torch.from_numpy(vel).cuda()
    sd = torch.from_numpy(initial_state(x, b.position)).cuda()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    colliders = b"".join(struct.pack(COLLIDER_FMT, c.type, *c.position, *c.half_extent, c.radius, c.friction,
                                     c.restitution) for c in scene.colliders)
    creation = struct.pack(jsb.CREATION_FMT, *b.creation)
    g = (ctypes.c_float * 3)(*scene.gravity)
    f = (ctypes.c_float * 3)(*b.force)
    torch.cuda.synchronize()
    for _ in range(steps):
        jsb.check(jsb.lib().jsb_step_body_noalloc(b.blob, len(b.blob), creation, colliders, len(scene.colliders), g, f,
                                                   scene.dt, xd.data_ptr(), vd.data_ptr(), sd.data_ptr(),
                                                   err.data_ptr(), None))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return sd.cpu().numpy()[:3], xd.cpu().numpy()[:, :3], vd.cpu().numpy()[:, :3]


def run_context(jsb, scene, body, steps):
    b = scene.bodies[body]
    ctx = jsb.Context(0)
    ctx.set_gravity(scene.gravity)
    for c in scene.colliders:
        ctx.add_collider(c.type, c.position, c.half_extent, c.radius, c.friction, c.restitution)
    bid = ctx.add_body(ctx.upload_settings(b.blob), b.creation, b.position)
    if any(v != 0.0 for v in b.force):
        ctx.set_step_force(bid, b.force)
    for _ in range(steps):
        ctx.step(scene.dt, 1)
    ctx.synchronize()
    out = ctx.read_body(bid)
    ctx.close()
    return out


@pytest.mark.parametrize("name,body", [("pinned_cloth", 0), ("uneven_small", 0), ("uneven_small", 7),
                                       ("diff_batch_small", 5), ("large_cloth_32", 0)])
def test_noalloc_matches_context_step(jsb, name, body):
    scene, _ = parse_scene(np.load(golden_path(name))["scene"].tobytes())
    got = run_noalloc(jsb, scene, body, 2)
    ref = run_context(jsb, scene, body, 2)
    for a, r, what in zip(got, ref, ("position", "local positions", "velocities")):
        assert np.array_equal(a, r), f"{what} differ: max {np.abs(a - r).max()}"


def test_noalloc_rejects_oversize_body(jsb):
    scene, _ = parse_scene(build_scene("large_cloth", n=136, steps=1))
    b = scene.bodies[0]
    assert b.num_vertices > 16384
    with pytest.raises(jsb.JsbError) as e:
        run_noalloc(jsb, scene, 0, 1)
    assert e.value.status == 8
    assert "16384" in str(e.value)


def test_noalloc_rejects_too_many_colliders(jsb):
    """More colliders than the fixed collider table holds (16) are refused before any device work."""
    scene, _ = parse_scene(np.load(golden_path("uneven_small"))["scene"].tobytes())
    scene.colliders = [scene.colliders[0]] * 17
    with pytest.raises(jsb.JsbError) as e:
        run_noalloc(jsb, scene, 0, 1)
    assert e.value.status == 8
    assert "16" in str(e.value)
