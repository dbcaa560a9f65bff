"""Dependency-level schedule invariants (host only).

The GPU projects all constraints of one level concurrently. That reproduces the reference's sequential
Gauss-Seidel order bit for bit iff (1) every constraint appears once, (2) for every vertex, a write
happens at a later level than every earlier access of that vertex in sequence order and a read happens
at a later level than the latest earlier write; the order inside a level is then irrelevant.
"""
import numpy as np
import pytest

from conftest import golden_path
from jsb_testlib import parse_scene

TYPE_BEND, TYPE_VOLUME, TYPE_EDGE, TYPE_LRA = 0, 1, 2, 3


def parse_constraints(blob):
    import struct
    off = 0
    out = {}
    for name, size in [("vertices", 28), ("faces", 16), ("edges", 16), ("bends", 24), ("volumes", 24),
                       ("skinned", 52), ("skinned_normals", 4), ("lras", 12), ("groups", 28)]:
        (n,) = struct.unpack_from("<I", blob, off)
        off += 4
        out[name] = np.frombuffer(blob, np.uint32, n * size // 4, off).reshape(n, size // 4) if n else np.zeros((0, size // 4), np.uint32)
        off += n * size
    return out


def sequence(c):
    """(type, index, written vertices, read-only vertices) in the reference's processing order."""
    seq = []
    prev = np.zeros(7, np.int64)
    for g in c["groups"].astype(np.int64):
        # group fields: edge, lra, rod_ss, rod_bt, bend, volume, skinned
        for i in range(prev[5], g[5]):
            seq.append((TYPE_VOLUME, i, tuple(c["volumes"][i, :4]), ()))
        for i in range(prev[4], g[4]):
            seq.append((TYPE_BEND, i, tuple(c["bends"][i, :4]), ()))
        for i in range(prev[0], g[0]):
            seq.append((TYPE_EDGE, i, tuple(c["edges"][i, :2]), ()))
        for i in range(prev[1], g[1]):
            seq.append((TYPE_LRA, i, (c["lras"][i, 1],), (c["lras"][i, 0],)))
        prev = g
    return seq


@pytest.mark.parametrize("name,body", [("pinned_cloth", 0), ("uneven_small", 0), ("uneven_small", 7),
                                       ("large_cloth_32", 0), ("diff_batch_small", 5)])
def test_levels_reproduce_sequential_order(jsb, name, body):
    scene, _ = parse_scene(np.load(golden_path(name))["scene"].tobytes())
    blob = scene.bodies[body].blob
    levels, records, source = jsb.settings_schedule(blob)
    c = parse_constraints(blob)
    seq = sequence(c)
    assert len(source) == len(seq)
    # level of every (type, index)
    level_of = {}
    L = len(levels) - 2
    for l in range(L):
        start, eb, ev, ee = levels[l]
        end = levels[l + 1][0]
        assert start <= eb <= ev <= ee <= end
        for k in range(start, end):
            t = int(source[k]) >> 28
            expect = TYPE_BEND if k < eb else TYPE_VOLUME if k < ev else TYPE_EDGE if k < ee else TYPE_LRA
            assert t == expect
            key = (t, int(source[k]) & 0x0FFFFFFF)
            assert key not in level_of
            level_of[key] = l
    assert len(level_of) == len(seq)
    last_write = {}
    max_access = {}
    for t, i, writes, reads in seq:
        l = level_of[(t, i)]
        for v in writes:
            assert l > max_access.get(v, -1)
        for v in reads:
            assert l > last_write.get(v, -1)
        for v in writes:
            last_write[v] = l
            max_access[v] = max(max_access.get(v, -1), l)
        for v in reads:
            max_access[v] = max(max_access.get(v, -1), l)
    # records carry the constraint data of their source
    for k in range(len(source)):
        t, i = int(source[k]) >> 28, int(source[k]) & 0x0FFFFFFF
        r = records[k]
        if t == TYPE_EDGE:
            e = c["edges"][i]
            assert r[0] == (e[0] | (e[1] << 16)) and r[2] == e[2] and r[3] == e[3]
        elif t == TYPE_BEND:
            b = c["bends"][i]
            assert r[0] == (b[0] | (b[1] << 16)) and r[1] == (b[2] | (b[3] << 16)) and r[2] == b[4] and r[3] == b[5]


def test_level_counts_pinned_cloth(jsb):
    """Schedule depth for the 30x30 pinned cloth (4 parallel groups + non-parallel group)."""
    scene, _ = parse_scene(np.load(golden_path("pinned_cloth"))["scene"].tobytes())
    levels, records, source = jsb.settings_schedule(scene.bodies[0].blob)
    L = len(levels) - 2
    assert len(source) == 3422 + 2465
    assert 100 < L < 600


TYPE_VERTEX = 4


def step_sequence(c, num_iterations):
    """The reference's whole-step order (type, index, substep, written, read): substep k's constraints,
    and before substeps 1.. each vertex's velocity update + integration (per-vertex passes)."""
    one = sequence(c)
    nv = len(c["vertices"])
    out = []
    for k in range(num_iterations):
        if k > 0:
            out += [(TYPE_VERTEX, v, k, (v,), ()) for v in range(nv)]
        out += [(t, i, k, w, r) for t, i, w, r in one]
    return out


@pytest.mark.parametrize("name,body", [("pinned_cloth", 0), ("uneven_small", 0), ("uneven_small", 7),
                                       ("large_cloth_32", 0), ("diff_batch_small", 5)])
def test_step_levels_reproduce_sequential_order(jsb, name, body):
    """Whole-step schedule: every constraint of every substep and every per-vertex pass between substeps
    appears once, typed as its level descriptor says, after every earlier access of its vertices."""
    scene, _ = parse_scene(np.load(golden_path(name))["scene"].tobytes())
    b = scene.bodies[body]
    n_it = b.num_iterations
    sched = jsb.settings_step_schedule(b.blob, n_it)
    assert sched is not None
    levels, records, source = sched
    c = parse_constraints(b.blob)
    seq = step_sequence(c, n_it)
    level_of = {}
    slot = 0
    for l, (start, bv, el, n) in enumerate(levels):
        assert start == slot
        ends = [bv & 0xFFFF, bv >> 16, el & 0xFFFF, el >> 16, n]
        assert all(e % 32 == 0 for e in ends) and ends == sorted(ends)
        for s in range(n):
            k = start + s
            src, sub = int(source[k, 0]), int(source[k, 1])
            if src == 0xFFFFFFFF:
                assert records[k, 0] == 0xFFFFFFFF
                continue
            t = src >> 28
            assert t == next(i for i, e in enumerate(ends) if s < e)
            key = (t, src & 0x0FFFFFFF, sub)
            assert key not in level_of
            level_of[key] = l
            if t == TYPE_VERTEX:
                assert records[k, 0] == (src & 0x0FFFFFFF)
        slot += n
    assert slot == len(source)
    assert len(level_of) == len(seq)
    last_write, max_access = {}, {}
    for t, i, k, writes, reads in seq:
        l = level_of[(t, i, k)]
        for v in writes:
            assert l > max_access.get(v, -1)
        for v in reads:
            assert l > last_write.get(v, -1)
        for v in writes:
            last_write[v] = l
            max_access[v] = max(max_access.get(v, -1), l)
        for v in reads:
            max_access[v] = max(max_access.get(v, -1), l)


def test_step_schedule_shortens_the_chain(jsb):
    """The 30x30 pinned cloth: the whole-step walk needs far fewer levels than 5 per-substep walks."""
    scene, _ = parse_scene(np.load(golden_path("pinned_cloth"))["scene"].tobytes())
    b = scene.bodies[0]
    per_substep = len(jsb.settings_schedule(b.blob)[0]) - 2
    levels, _, _ = jsb.settings_step_schedule(b.blob, b.num_iterations)
    assert len(levels) < 0.6 * b.num_iterations * per_substep
    assert jsb.settings_step_schedule(b.blob, 1) is None


def test_step_schedule_declines_levels_beyond_16_bits(jsb):
    """A level of 65,536 slots or more does not fit the packed level descriptor: the builder declines and
    the body walks every substep instead. Unconstrained vertices put all their per-vertex slots between
    substeps 0 and 1 into one level, padded to a multiple of 32: 65,505 of them need 65,536 slots,
    65,504 fit."""
    import struct

    def blob(nv):
        b = struct.pack("<I", nv) + struct.pack("<7f", 0, 0, 0, 0, 0, 0, 1.0) * nv
        b += struct.pack("<I", 0) * 5  # faces, edges, bends, volumes, skinned
        b += struct.pack("<I", 0) + struct.pack("<I", 0)  # skinned normals, LRA
        b += struct.pack("<I", 1) + struct.pack("<7I", 0, 0, 0, 0, 0, 0, 0)  # one (empty) update group
        b += struct.pack("<I", 0) * 3  # rods, inverse bind matrices
        return b

    assert jsb.settings_step_schedule(blob(65505), 2) is None
    levels, records, source = jsb.settings_step_schedule(blob(65504), 2)
    assert len(levels) == 1 and levels[0][3] == 65504 and (source[:, 0] >> 28 == 4).all()
