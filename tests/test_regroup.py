"""Opt-in regrouped settings (jsb_settings_regroup: a greedy colouring of each constraint type, one update
group; not the reference's order), host side: the bytes hold the same constraints, the remap says where
each came from, the dependency schedule is tens of levels per substep instead of hundreds to thousands,
and the oracle (which follows the reference's arithmetic for any valid settings) runs them stably, with
the deviation from the reference's order printed."""
import numpy as np

import joltphysics_gb300 as jsb
from jsb_testlib import blob_counts_py, parse_scene, rewrite_scene_blobs
from scenes import build_scene


def constraint_rows(blob):
    """Per type (edges, bends, volumes, LRA) the constraint records of a settings blob as byte rows."""
    off, out = 0, {}
    for name, size in (("v", 28), ("f", 16), ("e", 16), ("b", 24), ("vol", 24), ("sk", 52), ("skn", 4), ("lra", 12)):
        n = int(np.frombuffer(blob, np.uint32, 1, off)[0])
        out[name] = np.frombuffer(blob, np.uint8, n * size, off + 4).reshape(n, size)
        off += 4 + n * size
    return [out["e"], out["b"], out["vol"], out["lra"]]


def test_regrouped_bytes_hold_the_same_constraints():
    sc, _ = parse_scene(build_scene("uneven_batch", n_cloth=6, n_cube=4, cloth_max=24, cube_max=6))
    for b in sc.bodies:
        rb, remap = jsb.settings_regroup(b.blob)
        assert blob_counts_py(rb) == blob_counts_py(b.blob)
        old, new = constraint_rows(b.blob), constraint_rows(rb)
        k = 0
        for o, n in zip(old, new):
            m = remap[k:k + len(o)]
            k += len(o)
            assert sorted(m.tolist()) == list(range(len(o)))
            assert np.array_equal(n, o[m])
        assert k == len(remap)
        # every vertex (positions, masses) and face unchanged
        nv = b.num_vertices
        assert rb[:4 + 28 * nv] == b.blob[:4 + 28 * nv]


def test_regrouped_schedule_is_short():
    sc, _ = parse_scene(build_scene("large_cloth"))
    b = sc.bodies[0]
    rb, _ = jsb.settings_regroup(b.blob)
    lv0, _, _ = jsb.settings_schedule(b.blob)
    lv1, _, _ = jsb.settings_schedule(rb)
    print("256 x 256 cloth: levels per substep", len(lv0) - 2, "->", len(lv1) - 2)
    assert len(lv0) - 2 > 1000 and len(lv1) - 2 <= 40


def test_regrouped_pinned_cloth_runs_stably_in_the_oracle(oracle_lib):
    """Another Gauss-Seidel order changes the trajectory by a few percent of the motion (the hanging cloth's
    5 iterations do not converge its constraints; the order decides how stiffness spreads)."""
    scene_bytes = build_scene("pinned_cloth", steps=60)
    rscene_bytes = rewrite_scene_blobs(scene_bytes, lambda blob: jsb.settings_regroup(blob)[0])
    runs, start = [], None
    for sb in (scene_bytes, rscene_bytes):
        scene, _ = parse_scene(sb)
        o = oracle_lib(scene)
        pos, loc, _ = o.body(0)
        start = pos + loc
        o.step(60)
        pos, loc, vel = o.body(0)
        runs.append(pos + loc)
    dev = np.abs(runs[0] - runs[1]).max()
    moved = np.abs(runs[0] - start).max()
    print("pinned 30 x 30 cloth, 60 steps: max |x(regrouped) - x(reference order)| = %.3e m, max motion %.3e m" % (dev, moved))
    assert np.isfinite(runs[1]).all() and dev <= 0.1 * moved
