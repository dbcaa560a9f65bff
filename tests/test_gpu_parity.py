"""GPU solver parity through the C ABI.

Bar: bitwise equality with the reference (golden fixtures written by the reference built with
JPH_CROSS_PLATFORM_DETERMINISTIC) and with the CPU oracle on the same inputs. Body positions, local
vertex positions and velocities are compared exactly. At full workload sizes, where the oracle is too
slow for every step, size-independent properties are checked (determinism, plain == batched == graph,
finite state, kinematic vertices fixed in world space).
"""
import numpy as np
import pytest

from conftest import golden_path
from jsb_testlib import Oracle, parse_scene
from scenes import build_scene

pytestmark = pytest.mark.gpu

GOLDEN = ["pinned_cloth", "uneven_small", "large_cloth_32", "diff_cloth_16", "diff_batch_small", "sleep_small", "shapes_drop"]


def split(arr, nv):
    out, off = [], 0
    for n in nv:
        out.append(arr[off:off + n])
        off += n
    return out


def make_ctx(jsb, scene_bytes, step_forces=False):
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    if step_forces:
        ctx.set_scene_step_forces()
    return ctx


def advance(ctx, n, mode="batched"):
    if n <= 0:
        return
    if mode == "graph":
        ctx.step_graph(n, 1)
        return
    for _ in range(n):
        if mode == "plain":
            ctx.step_plain()
        else:
            ctx.step()


def snapshot(ctx):
    ctx.synchronize()
    return [ctx.read_body(b["id"]) for b in ctx.bodies]


def assert_same(a, b, what):
    for i, (x, y) in enumerate(zip(a, b)):
        for k, name in enumerate(("position", "local", "velocity")):
            assert np.array_equal(x[k], y[k]), f"{what}: body {i} {name} differs, max {np.abs(x[k] - y[k]).max()}"


@pytest.mark.parametrize("name", GOLDEN)
def test_bitwise_vs_reference(jsb, name):
    g = np.load(golden_path(name))
    nv = list(g["num_vertices"])
    ctx = make_ctx(jsb, g["scene"].tobytes(), step_forces=True)
    cur = 0
    for step in g["steps"]:
        advance(ctx, int(step) - cur)
        cur = int(step)
        snap = snapshot(ctx)
        ref = [(g[f"det_pos_{step}"][b], split(g[f"det_local_{step}"], nv)[b], split(g[f"det_vel_{step}"], nv)[b])
               for b in range(len(nv))]
        assert_same(snap, ref, f"{name} step {step}")
        if f"det_timer_{step}" in g:  # sleep timers in the SaveState bytes, and which bodies sleep
            for b in range(len(nv)):
                timer = np.frombuffer(ctx.save_state(b), np.float32, 1, 96)[0]
                assert timer == g[f"det_timer_{step}"][b], (name, step, b, timer)
                assert ctx.is_active(b) == bool(timer < 0.5), (name, step, b)


def test_pinned_cloth_tolerance_vs_fma_reference(jsb):
    """Stated bar: <= 1e-5 m after 1 step and <= 1e-3 m after 300 steps against the default build too."""
    g = np.load(golden_path("pinned_cloth"))
    ctx = make_ctx(jsb, g["scene"].tobytes())
    advance(ctx, 300)
    pos, loc, _ = snapshot(ctx)[0]
    world = loc.astype(np.float64) + pos
    ref = g["fast_local_300"].astype(np.float64) + g["fast_pos_300"][0]
    assert np.abs(world - ref).max() <= 1e-3


@pytest.mark.parametrize("mode", ["plain", "graph"])
def test_plain_and_graph_equal_batched(jsb, mode):
    g = np.load(golden_path("diff_batch_small"))
    a = make_ctx(jsb, g["scene"].tobytes(), step_forces=True)
    b = make_ctx(jsb, g["scene"].tobytes(), step_forces=True)
    advance(a, 12, "batched")
    advance(b, 12, mode)
    assert_same(snapshot(a), snapshot(b), mode)


def test_full_size_bodies_vs_oracle(jsb):
    """Full cloth/cube size ranges of the uneven batch (cloth sides 8..64, cubes 4..12 cells)."""
    scene_bytes = build_scene("uneven_batch", n_cloth=24, n_cube=8, steps=4)
    scene, _ = parse_scene(scene_bytes)
    o = Oracle(scene)
    ctx = make_ctx(jsb, scene_bytes)
    for s in range(3):
        o.step(1)
        advance(ctx, 1)
        ref = [o.body(i) for i in range(len(scene.bodies))]
        assert_same(snapshot(ctx), ref, f"step {s + 1}")


def test_diff_batch_full_vs_oracle(jsb):
    """256-body differentiable batch (forces every step, pressure, floor + sphere) for 2 steps."""
    scene_bytes = build_scene("diff_batch", steps=2)
    scene, _ = parse_scene(scene_bytes)
    o = Oracle(scene)
    ctx = make_ctx(jsb, scene_bytes, step_forces=True)
    o.step(2)
    advance(ctx, 2)
    assert_same(snapshot(ctx), [o.body(i) for i in range(len(scene.bodies))], "diff_batch")


def test_uneven_batch_full_properties(jsb):
    """The full 512-body uneven batch: two runs are bitwise identical, the first step matches the oracle,
    everything stays finite and kinematic vertices stay put in world space."""
    scene_bytes = build_scene("uneven_batch")
    scene, _ = parse_scene(scene_bytes)
    o = Oracle(scene)
    o.step(1)
    a = make_ctx(jsb, scene_bytes)
    init = snapshot(a)
    advance(a, 1)
    assert_same(snapshot(a), [o.body(i) for i in range(len(scene.bodies))], "uneven_batch step 1")
    advance(a, 29, "graph")
    sa = snapshot(a)
    b = make_ctx(jsb, scene_bytes)
    advance(b, 30)
    assert_same(sa, snapshot(b), "determinism")
    for i, (pos, loc, vel) in enumerate(sa):
        assert np.isfinite(loc).all() and np.isfinite(vel).all()
    # kinematic (pinned) cloth rows stay fixed in world space
    from jsb_testlib import blob_num_vertices
    import struct
    for i, body in enumerate(scene.bodies[:16]):
        n = body.num_vertices
        inv_mass = np.frombuffer(body.blob, np.float32, 7 * n, 4).reshape(n, 7)[:, 6]
        pinned = inv_mass == 0
        w0 = init[i][1].astype(np.float64) + init[i][0]
        w1 = sa[i][1].astype(np.float64) + sa[i][0]
        assert np.abs(w1[pinned] - w0[pinned]).max() < 1e-4


def test_save_restore_roundtrip(jsb):
    g = np.load(golden_path("uneven_small"))
    a = make_ctx(jsb, g["scene"].tobytes())
    advance(a, 5)
    states = [a.save_state(b["id"]) for b in a.bodies]
    positions = [s[0] for s in snapshot(a)]
    b = make_ctx(jsb, g["scene"].tobytes())
    for body, st, pos in zip(b.bodies, states, positions):
        b.restore_state(body["id"], st, pos)
    assert_same(snapshot(a), snapshot(b), "restore")
    advance(a, 5)
    advance(b, 5)
    assert_same(snapshot(a), snapshot(b), "after restore")


def test_host_buffer_roundtrip(jsb):
    g = np.load(golden_path("uneven_small"))
    a = make_ctx(jsb, g["scene"].tobytes())
    advance(a, 3)
    n = a.total_vertices()
    pos = np.zeros((n, 3), np.float32)
    vel = np.zeros((n, 3), np.float32)
    a.download_all(pos, vel)
    a.synchronize()
    before = snapshot(a)
    a.upload_all(pos, vel)
    a.synchronize()
    assert_same(before, snapshot(a), "host round trip")


def test_nonfinite_state_reported(jsb):
    g = np.load(golden_path("pinned_cloth"))
    a = make_ctx(jsb, g["scene"].tobytes())
    st = bytearray(a.save_state(0))
    # first vertex position x := NaN (101-byte motion header, then position/velocity per vertex)
    st[101:105] = np.array([np.nan], np.float32).tobytes()
    a.restore_state(0, bytes(st), (0.0, 10.0, 0.0))
    a.step()
    with pytest.raises(jsb.JsbError) as e:
        a.synchronize()
    assert e.value.status == 7


@pytest.mark.parametrize("path", ["one_cta", "cluster"])
def test_nan_propagation_matches_oracle(jsb, path):
    """A body holding NaN positions (as a body that has blown up does) keeps being stepped: the vertices
    that become NaN are those that become NaN in the reference's arithmetic (NaN-guarded projections),
    and the other bodies are untouched, bit for bit."""
    scene_bytes = build_scene("uneven_batch", n_cloth=4, n_cube=0, cloth_max=24, steps=3, seed=9)
    scene, _ = parse_scene(scene_bytes)
    ctx = make_ctx(jsb, scene_bytes)
    if path == "cluster":
        for mv, t, _ in ctx.bucket_table():
            ctx.set_bucket_config(mv, t, 2)
    n = ctx.total_vertices()
    pos = np.zeros((n, 3), np.float32)
    vel = np.zeros((n, 3), np.float32)
    ctx.download_all(pos, vel)
    ctx.synchronize()
    nv = [b.num_vertices for b in scene.bodies]
    poisoned = 0  # a cloth: a few vertices in its interior
    off = 0
    idx = [nv[poisoned] // 2, nv[poisoned] // 2 + 1, nv[poisoned] // 3]
    pos[[off + i for i in idx], 1] = np.nan
    ctx.upload_all(pos, vel)
    o = Oracle(scene)
    offs = np.concatenate([[0], np.cumsum(nv)])
    for b in range(len(nv)):
        o.set_state(b, pos[offs[b]:offs[b + 1]], vel[offs[b]:offs[b + 1]])
    for step in range(3):
        o.step(1)
        ctx.step()
        with pytest.raises(jsb.JsbError):
            ctx.synchronize()
        snap = snapshot(ctx)
        for b in range(len(nv)):
            ref = o.body(b)
            if b == poisoned:
                gm, rm = np.isnan(snap[b][1]), np.isnan(ref[1])
                assert np.array_equal(gm, rm), (step, int(gm.sum()), int(rm.sum()), np.isnan(snap[b][0]), np.isnan(ref[0]),
                                                 np.argwhere(gm != rm)[:6].tolist(), int(np.isnan(snap[b][2]).sum()),
                                                 int(np.isnan(ref[2]).sum()))
                assert gm.any()
            else:
                for k in range(3):
                    assert np.array_equal(snap[b][k], ref[k]), (b, k)


@pytest.mark.parametrize("state_mode,threads", [(0, 0), (1, 0), (0, 512), (1, 512)])
def test_step_walk_equals_substep_walk_and_oracle(jsb, state_mode, threads):
    """Whole-step walk (default) against the per-substep walk and the oracle, through contact: bodies of
    the uneven batch's full size ranges drop onto the floor (cubes land, pinned cloths hang), 90
    steps; state_mode 1 keeps velocities and previous positions in HBM, which the per-vertex passes
    inside the walk then read and write there; threads 512 (else the default table's) per CTA."""
    scene_bytes = build_scene("uneven_batch", n_cloth=10, n_cube=6, steps=90, seed=11)
    scene, _ = parse_scene(scene_bytes)
    a = make_ctx(jsb, scene_bytes)
    b = jsb.Context(0)
    b.set_step_walk(False)
    b.load_scene(scene_bytes)
    for ctx in (a, b):
        for mv, t, _ in ctx.bucket_table():
            ctx.set_bucket_config(mv, threads or t, state_mode)
    o = Oracle(scene)
    cur = 0
    for step in (1, 45, 90):
        advance(a, step - cur)
        advance(b, step - cur, "graph")
        o.step(step - cur)
        cur = step
        sa = snapshot(a)
        assert_same(sa, snapshot(b), f"step walk vs substep walk, step {step}")
        assert_same(sa, [o.body(i) for i in range(len(scene.bodies))], f"step walk vs oracle, step {step}")
    # the floor was reached: some vertex of a cube sits on it
    assert min((loc[:, 1] + pos[1]).min() for pos, loc, _ in sa[10:]) < 0.05


def test_sleeping_body_wakes_on_force(jsb):
    """A body asleep on the floor is not stepped (its state stays bit for bit); AddForce wakes it and
    restarts its sleep timer (BodyInterface::AddForce with EActivation::Activate), like the oracle."""
    g = np.load(golden_path("sleep_small"))
    scene_bytes = g["scene"].tobytes()
    scene, _ = parse_scene(scene_bytes)
    ctx = make_ctx(jsb, scene_bytes)
    o = Oracle(scene)
    advance(ctx, 160, "graph")
    o.step(160)
    asleep = [b for b in range(len(scene.bodies)) if not ctx.is_active(b)]
    assert asleep and all(not o.active(b) for b in asleep)
    before = snapshot(ctx)
    advance(ctx, 5)
    after = snapshot(ctx)
    for b in asleep:
        for k in range(3):
            assert np.array_equal(before[b][k], after[b][k])
    o.step(5)
    b = asleep[0]
    ctx.add_force(b, (0.0, 50.0, 0.0))
    scene.bodies[b].force = (0.0, 50.0, 0.0)  # the oracle applies the force before its next step
    o.step(1)
    scene.bodies[b].force = (0.0, 0.0, 0.0)
    ctx.step()
    assert ctx.is_active(b) and o.active(b)
    assert_same(snapshot(ctx), [o.body(i) for i in range(len(scene.bodies))], "after the wake")
    o.step(3)
    advance(ctx, 3)
    assert_same(snapshot(ctx), [o.body(i) for i in range(len(scene.bodies))], "3 steps later")
