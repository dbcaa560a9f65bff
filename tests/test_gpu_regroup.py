"""Opt-in regrouped settings (jsb_settings_regroup; not the reference's constraint order) on the GPU.

The regrouped bytes are ordinary settings with one update group, so the GPU walks their (much shorter)
dependency schedule with the same kernels, and the CPU oracle runs their sequential order. Bar: bitwise
equality with the oracle on the regrouped settings, on the one-CTA path (a batch slice with cloths and
pressurised cubes, floor contact) and on the cluster path (the 256 x 256 cloth); the deviation from the
reference's order is measured in tests/test_regroup.py and reported by bench.py.
"""
import os

import numpy as np
import pytest

import joltphysics_gb300 as jsb_mod
from jsb_testlib import Oracle, parse_scene, rewrite_scene_blobs
from test_gpu_parity import advance, assert_same, make_ctx, snapshot
from scenes import build_scene

pytestmark = pytest.mark.gpu


def regrouped(scene_bytes):
    return rewrite_scene_blobs(scene_bytes, lambda blob: jsb_mod.settings_regroup(blob)[0])


def test_regrouped_batch_slice_vs_oracle(jsb):
    scene_bytes = regrouped(build_scene("uneven_batch", n_cloth=10, n_cube=6, cloth_max=32, cube_max=7, steps=60))
    scene, _ = parse_scene(scene_bytes)
    ctx = make_ctx(jsb, scene_bytes)
    o = Oracle(scene, threads=os.cpu_count() or 1)
    for k in range(3):
        o.step(20)
        advance(ctx, 20)
        assert_same(snapshot(ctx), [o.body(b) for b in range(len(scene.bodies))], f"step {20 * (k + 1)}")


def test_regrouped_large_cloth_cluster_path_vs_oracle(jsb):
    scene_bytes = regrouped(build_scene("large_cloth", n=256, steps=3))
    scene, _ = parse_scene(scene_bytes)
    ctx = make_ctx(jsb, scene_bytes)
    cfg = ctx.cluster_config()
    assert cfg["bodies"] == 1, cfg
    o = Oracle(scene, threads=os.cpu_count() or 1)
    for s in range(2):
        o.step(1)
        advance(ctx, 1)
        assert_same(snapshot(ctx), [o.body(0)], f"step {s + 1}")
