"""Thread-block-cluster path (bodies spread over the shared memory of a cluster) through the C ABI.

Bar: bitwise equality with the CPU oracle (itself bitwise equal to the reference built with
JPH_CROSS_PLATFORM_DETERMINISTIC) and with the one-CTA path, for every cluster shape. The 256 x 256
cloth (65,536 vertices, LRA tethers, sphere + floor) only fits this path.
"""
import os

import numpy as np
import pytest

from jsb_testlib import Oracle, parse_scene
from test_gpu_parity import advance, assert_same, make_ctx, snapshot
from scenes import build_scene

pytestmark = pytest.mark.gpu


def force_cluster(ctx, cluster_size=0, threads=256):
    """Send every bucket's bodies to the cluster path."""
    for mv, t, _ in ctx.bucket_table():
        ctx.set_bucket_config(mv, t, 2)
    ctx.set_cluster_config(cluster_size, threads)


def test_large_cloth_65536_vertices_vs_oracle(jsb):
    scene_bytes = build_scene("large_cloth", n=256, steps=3)
    scene, _ = parse_scene(scene_bytes)
    ctx = make_ctx(jsb, scene_bytes)
    cfg = ctx.cluster_config()
    assert cfg["bodies"] == 1 and cfg["cluster_size"] >= 8, cfg
    o = Oracle(scene, threads=os.cpu_count() or 1)
    for s in range(2):
        o.step(1)
        advance(ctx, 1)
        assert_same(snapshot(ctx), [o.body(0)], f"step {s + 1}")


@pytest.mark.parametrize("cluster_size,threads", [(2, 128), (4, 512), (8, 256), (16, 256), (16, 512)])
def test_cluster_shapes_vs_oracle_through_contact(jsb, cluster_size, threads):
    """A 48 x 48 cloth dropped onto the sphere: 40 steps cover the first contacts."""
    scene_bytes = build_scene("large_cloth", n=48, steps=40)
    scene, _ = parse_scene(scene_bytes)
    ctx = make_ctx(jsb, scene_bytes)
    force_cluster(ctx, cluster_size, threads)
    assert ctx.cluster_config() == {"cluster_size": cluster_size, "threads": threads, "bodies": 1}
    o = Oracle(scene)
    o.step(40)
    advance(ctx, 40)
    assert_same(snapshot(ctx), [o.body(0)], f"cluster {cluster_size} x {threads}")


def test_cluster_equals_one_cta_path_on_a_batch(jsb):
    """Cloths of many sizes (no pressure), floor contact: cluster path == one-CTA path, bitwise, in the
    batched, plain and graph forms."""
    scene_bytes = build_scene("uneven_batch", n_cloth=12, n_cube=0, steps=30, seed=9)
    a = make_ctx(jsb, scene_bytes)
    advance(a, 30)
    for mode in ("batched", "plain", "graph"):
        b = make_ctx(jsb, scene_bytes)
        force_cluster(b)
        assert b.cluster_config()["bodies"] == 12
        advance(b, 30, mode)
        assert_same(snapshot(a), snapshot(b), f"cluster path ({mode})")


def test_mixed_launch_cluster_and_one_cta_bodies(jsb):
    """A context holding a 65,536-vertex cloth and small bodies runs both paths in one batched step."""
    big = build_scene("large_cloth", n=256, steps=2)
    small = build_scene("uneven_batch", n_cloth=6, n_cube=3, steps=2, seed=4)
    ctx = make_ctx(jsb, big)
    ctx.load_scene(small)
    assert ctx.cluster_config()["bodies"] == 1
    scene, _ = parse_scene(big)
    s2, _ = parse_scene(small)
    scene.colliders += s2.colliders
    scene.bodies += s2.bodies
    o = Oracle(scene, threads=os.cpu_count() or 1)
    o.step(2)
    advance(ctx, 2)
    assert_same(snapshot(ctx), [o.body(i) for i in range(len(scene.bodies))], "cluster and one-CTA bodies")


@pytest.mark.parametrize("cluster_size,threads", [(2, 128), (4, 256), (16, 256)])
def test_pressurised_bodies_on_cluster_path_vs_oracle(jsb, cluster_size, threads):
    """Pressurised tet cubes (with unpressurised ones) forced onto the cluster path: ApplyPressure's face
    terms dealt over the cluster and summed in face order; bitwise equal to the oracle through the floor
    contact."""
    scene_bytes = build_scene("uneven_batch", n_cloth=0, n_cube=8, cube_max=7, steps=40, seed=3)
    scene, _ = parse_scene(scene_bytes)
    assert any(float(b.creation[5]) > 0.0 for b in scene.bodies), "no pressurised cube drawn"
    ctx = make_ctx(jsb, scene_bytes)
    force_cluster(ctx, cluster_size, threads)
    o = Oracle(scene, threads=os.cpu_count() or 1)
    for k in range(2):
        o.step(20)
        advance(ctx, 20)
        assert_same(snapshot(ctx), [o.body(b) for b in range(len(scene.bodies))], f"step {20 * (k + 1)}")


def test_cluster_config_validation(jsb):
    ctx = jsb.Context(0)
    for size, threads in ((3, 256), (32, 256), (8, 64), (8, 1024)):
        with pytest.raises(jsb.JsbError) as e:
            ctx.set_cluster_config(size, threads)
        assert e.value.status == jsb.JSB_ERR_INVALID_ARGUMENT
    ctx.set_cluster_config(0, 512)
    assert ctx.cluster_config() == {"cluster_size": 0, "threads": 512, "bodies": 0}
    ctx.close()


def test_contact_readback_cluster_equals_one_cta_path(jsb):
    """SoftBodyManifold readback (jsb_body_contacts) on the cluster path equals the one-CTA path's (itself
    checked against the reference's manifolds), bitwise: cloths and cubes (some pressurised) dropped onto a
    capsule, two cylinders, a sphere and the floor."""
    scene_bytes = build_scene("shapes_drop", steps=60)
    a, b = make_ctx(jsb, scene_bytes), make_ctx(jsb, scene_bytes)
    force_cluster(b, 2, 128)
    for c in (a, b):
        c.set_contact_readback(True)
    touched = 0
    for step in range(60):
        advance(a, 1)
        advance(b, 1)
        for body in range(len(a.bodies)):
            ca, cb = a.contacts(body), b.contacts(body)
            for k in ("has_contact", "points", "normals", "shape", "delta"):
                assert np.array_equal(ca[k], cb[k]), (step, body, k)
            touched += int(ca["has_contact"].sum())
    assert touched > 100, touched
