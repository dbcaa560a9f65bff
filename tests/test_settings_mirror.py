"""The library's SoftBodySharedSettings mirror (CreateConstraints + Optimize + SaveBinaryState) against
the bytes Jolt itself wrote for the same seeded scenes."""
import numpy as np
import pytest

from conftest import golden_path
from scenes import build_scene

CASES = {
    "pinned_cloth": ("pinned_cloth", {}),
    "uneven_small": ("uneven_batch", dict(n_cloth=6, n_cube=3, cloth_max=20, cube_max=5, steps=40)),
    "large_cloth_32": ("large_cloth", dict(n=32, steps=120)),
    "diff_cloth_16": ("diff_cloth", dict(n=16, steps=40)),
    "diff_batch_small": ("diff_batch", dict(n_cloth=4, n_cube=2, steps=30)),
    "sleep_small": ("uneven_batch", dict(n_cloth=6, n_cube=3, cloth_max=20, cube_max=5, steps=200, sleep=1)),
    "shapes_drop": ("shapes_drop", {}),
}


@pytest.mark.parametrize("name", list(CASES))
def test_mirror_bytes_equal_reference(name, jsb):
    scene, params = CASES[name]
    mine = build_scene(scene, **params)
    ref = np.load(golden_path(name))["scene"].tobytes()
    assert mine == ref
