"""The C ABI library: it loads, exports every entry point include/jsb.h declares, and rejects malformed
settings bytes with the documented status codes (host-only calls; no device needed)."""
import os
import re
import struct

import numpy as np
import pytest

from conftest import REPO, golden_path
from jsb_testlib import parse_scene


def declared_functions():
    text = open(os.path.join(REPO, "include", "jsb.h")).read()
    return sorted(set(re.findall(r"^\s*(?:jsb_status|const char \*)\s*(jsb_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(jsb):
    names = declared_functions()
    assert len(names) >= 20
    L = jsb.lib()
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(jsb.SIGNATURES), set(names) ^ set(jsb.SIGNATURES)


def pinned_blob():
    scene, _ = parse_scene(np.load(golden_path("pinned_cloth"))["scene"].tobytes())
    return scene.bodies[0].blob


def status_of(jsb, blob):
    try:
        jsb.settings_schedule(blob)
        return 0
    except jsb.JsbError as e:
        return e.status


def test_truncated_blob_rejected(jsb):
    blob = pinned_blob()
    assert status_of(jsb, blob) == 0
    for cut in (0, 3, 100, len(blob) // 2, len(blob) - 1):
        assert status_of(jsb, blob[:cut]) == 2, cut
    assert status_of(jsb, blob + b"\0") == 2


def test_out_of_range_index_rejected(jsb):
    blob = bytearray(pinned_blob())
    nv = struct.unpack_from("<I", blob, 0)[0]
    off = 4 + 28 * nv
    nf = struct.unpack_from("<I", blob, off)[0]
    off += 4 + 16 * nf
    # first edge's first vertex
    struct.pack_into("<I", blob, off + 4, nv + 5)
    assert status_of(jsb, bytes(blob)) == 2


def _sections(blob):
    """Byte offsets of the count fields of each SaveBinaryState section."""
    sizes = [28, 16, 16, 24, 24, 52, 4, 12, 28, 36, 28, 68]
    offs, off = [], 0
    for s in sizes:
        offs.append(off)
        (n,) = struct.unpack_from("<I", blob, off)
        off += 4 + n * s
    return offs


def test_unsupported_rods_and_missing_groups(jsb):
    blob = pinned_blob()
    offs = _sections(blob)
    # append one rod stretch-shear constraint (36 bytes) and make the last group cover it
    rod_off = offs[9]
    rod = struct.pack("<2I3f4f", 0, 1, 1.0, 1.0, 0.0, 0, 0, 0, 1)
    b = bytearray(blob[:rod_off]) + struct.pack("<I", 1) + rod + blob[rod_off + 4:]
    groups_off = offs[8]
    (ng,) = struct.unpack_from("<I", b, groups_off)
    struct.pack_into("<I", b, groups_off + 4 + 28 * (ng - 1) + 8, 1)
    assert status_of(jsb, bytes(b)) == 3
    # no update groups: Optimize was not called
    (ng,) = struct.unpack_from("<I", blob, groups_off)
    b2 = blob[:groups_off] + struct.pack("<I", 0) + blob[groups_off + 4 + 28 * ng:]
    assert status_of(jsb, b2) == 2


def test_context_without_gpu_fails_cleanly(jsb):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(jsb.JsbError) as e:
        jsb.Context(0)
    assert e.value.status == 4
