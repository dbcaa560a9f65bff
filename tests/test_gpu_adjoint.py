"""Hand-written adjoint of the GPU step against FP64 references.

The loss is a random linear functional of world positions after chosen steps. Two references:
  * FP64 central finite differences of the CPU oracle (its double-precision evaluation of the same
    constraint order) for a random sample of parameters: initial positions, initial velocities,
    per-edge and per-volume compliance and step force;
  * the gradient of a plain FP64 torch re-implementation of the step (tests/torch_ref.py) by autodiff,
    for every parameter, with the collision active set frozen like the adjoint.
Bar: relative error of each parameter kind's gradient vector, ||g - g_ref|| / ||g_ref|| <= 1e-3.
The GPU adjoint linearises the FP32 trajectory, the references the FP64 one. Without contacts the two
stay close enough for the 1e-3 bar against finite differences; through contact events the autodiff
reference is also evaluated along the GPU trajectory (state pinned after every step), where the bar holds
for every parameter kind, and the free-running gap is bounded separately.
"""
import numpy as np
import pytest

from jsb_testlib import FD64, parse_scene
from scenes import build_scene

pytestmark = pytest.mark.gpu

EPS = {"x0": 1e-6, "v0": 1e-6, "force": 1e-6}


def gpu_gradients(jsb, scene_bytes, seeds, steps, every, forces=None, trajectory=None, step_walk=True):
    """Adjoint gradients per body; fills `trajectory[step][body] = (world positions, velocities)` if given."""
    ctx = jsb.Context(0)
    ctx.set_step_walk(step_walk)
    ctx.load_scene(scene_bytes)
    ctx.set_scene_step_forces()
    for b, f in (forces or {}).items():
        ctx.set_step_force(b, f)
    ctx.adjoint_begin(steps, every)
    if trajectory is None:
        ctx.adjoint_forward()
    else:
        for s in range(1, steps + 1):
            ctx.adjoint_forward(s)
            trajectory[s] = []
            for b in range(len(ctx.bodies)):
                pos, loc, vel = ctx.read_body(b)
                trajectory[s].append((loc.astype(np.float64) + pos.astype(np.float64), vel.astype(np.float64)))
    for step, per_body in seeds.items():
        for b, r in per_body.items():
            ctx.adjoint_seed(step, b, r.astype(np.float32))
    ctx.adjoint_backward()
    out = [ctx.adjoint_gradients(b["id"], b["num_edges"], b["num_volumes"]) for b in ctx.bodies]
    ctx.adjoint_end()
    ctx.close()
    return out


def sample_and_compare(fd, grads, picks, rng, frozen=False):
    errors = []
    for body, kind, count in picks:
        base = fd.base_params(body)[kind]
        g = grads[body]
        key = {"x0": "x0", "v0": "v0", "edge": "edge_compliance", "volume": "volume_compliance", "force": "force"}[kind]
        gpu = g[key]
        idxs = [tuple(np.unravel_index(rng.integers(base.size), base.shape)) for _ in range(count)]
        fds, gps = [], []
        for idx in idxs:
            eps = EPS.get(kind, 1e-6 * abs(base[idx]) + 1e-14)
            fds.append(fd.central(body, kind, idx, eps, frozen=frozen))
            gps.append(float(gpu[idx]))
        fds, gps = np.array(fds), np.array(gps)
        rel = np.linalg.norm(gps - fds) / max(np.linalg.norm(fds), 1e-30)
        errors.append((kind, body, rel, fds, gps))
    return errors


def test_adjoint_cloth_vs_fd(jsb):
    scene_bytes = build_scene("diff_cloth", n=10, steps=16)
    scene, _ = parse_scene(scene_bytes)
    rng = np.random.default_rng(7)
    nv = scene.bodies[0].num_vertices
    seeds = {8: {0: rng.standard_normal((nv, 3))}, 16: {0: rng.standard_normal((nv, 3))}}
    force = {0: np.array([0.3, -0.2, 0.1], np.float32)}
    grads = gpu_gradients(jsb, scene_bytes, seeds, 16, 5, force)
    fd = FD64(scene, seeds, 16)
    scene.bodies[0].force = tuple(float(v) for v in force[0])
    errs = sample_and_compare(fd, grads, [(0, "x0", 10), (0, "v0", 10), (0, "edge", 9), (0, "force", 3)], rng)
    for kind, body, e, fds, gps in errs:
        print(kind, body, "rel", e, "\n  fd ", fds, "\n  gpu", gps)
    assert max(e for _, _, e, _, _ in errs) <= 1e-3, [(k, e) for k, _, e, _, _ in errs]


def test_adjoint_cloth_with_bends_vs_fd(jsb):
    """A 10 x 10 cloth with dihedral bends (flat at the start: the bend adjoint goes through the signed
    angle, bounded at flat pairs), 16 steps: positions, velocities, edge compliances and force against
    FP64 central differences, and bend compliances against FP64 autodiff (pinned to the GPU trajectory),
    1e-3."""
    from torch_ref import reference_gradients

    scene_bytes = build_scene("diff_cloth", n=10, steps=16, bends=1)
    scene, _ = parse_scene(scene_bytes)
    rng = np.random.default_rng(9)
    nv = scene.bodies[0].num_vertices
    seeds = {8: {0: rng.standard_normal((nv, 3))}, 16: {0: rng.standard_normal((nv, 3))}}
    force = {0: np.array([0.3, -0.2, 0.1], np.float32)}
    traj = {}
    grads = gpu_gradients(jsb, scene_bytes, seeds, 16, 5, force, trajectory=traj)
    scene.bodies[0].force = tuple(float(v) for v in force[0])
    fd = FD64(scene, seeds, 16)
    errs = sample_and_compare(fd, grads, [(0, "x0", 10), (0, "v0", 10), (0, "edge", 9), (0, "force", 3)], rng)
    for kind, body, e, fds, gps in errs:
        print(kind, body, "rel", e, "\n  fd ", fds, "\n  gpu", gps)
    assert max(e for _, _, e, _, _ in errs) <= 1e-3, [(k, e) for k, _, e, _, _ in errs]
    ctx = jsb.Context(0)  # bend compliance gradients of the same run
    ctx.load_scene(scene_bytes)
    ctx.set_step_force(0, force[0])
    ctx.adjoint_begin(16, 5)
    ctx.adjoint_forward()
    for step, per_body in seeds.items():
        ctx.adjoint_seed(step, 0, per_body[0].astype(np.float32))
    ctx.adjoint_backward()
    from jsb_testlib import blob_bend_compliance

    gb = ctx.adjoint_bend_gradients(0, len(blob_bend_compliance(scene.bodies[0].blob))).astype(np.float64)
    ctx.adjoint_end()
    ctx.close()
    ref, _ = reference_gradients(scene, seeds, 16, traj)
    e = np.linalg.norm(gb - ref[0]["bend"]) / np.linalg.norm(ref[0]["bend"])
    print("bend compliance rel", e)
    assert e <= 1e-3, e


def contact_scene(jsb):
    """A cloth and a pressurised tet cube dropped 0.15 m onto the floor, with step forces."""
    return build_scene("diff_batch", n_cloth=1, n_cube=1, steps=24, drop_mm=150, seed=23)


def test_adjoint_contacts_vs_fp64_autodiff(jsb):
    from torch_ref import reference_gradients

    scene_bytes = contact_scene(jsb)
    scene, _ = parse_scene(scene_bytes)
    rng = np.random.default_rng(11)
    seeds = {24: {b: rng.standard_normal((body.num_vertices, 3)) for b, body in enumerate(scene.bodies)},
             12: {1: rng.standard_normal((scene.bodies[1].num_vertices, 3))}}
    traj = {}
    grads = gpu_gradients(jsb, scene_bytes, seeds, 24, 8, trajectory=traj)
    worst = {}
    for label, pin in (("pinned", traj), ("free", None)):
        ref, _ = reference_gradients(scene, seeds, 24, pin)
        worst[label] = 0.0
        for b in range(len(scene.bodies)):
            for key, rkey in (("x0", "x0"), ("v0", "v0"), ("force", "force"), ("edge_compliance", "edge"),
                              ("volume_compliance", "volume")):
                g, r = grads[b][key].astype(np.float64).ravel(), np.asarray(ref[b][rkey]).ravel()
                if r.size == 0 or np.linalg.norm(r) == 0:
                    continue
                err = np.abs(g - r)
                e = np.linalg.norm(g - r) / np.linalg.norm(r)
                top = np.argsort(err)[-3:]
                print(f"{label} body {b} {key}: rel {e:.3e} (|ref| {np.linalg.norm(r):.3e}) worst idx {top} "
                      f"gpu {g[top]} ref {r[top]}")
                worst[label] = max(worst[label], e)
    # Along the GPU's own trajectory the adjoint is the FP64 derivative up to FP32 rounding of the sweep.
    assert worst["pinned"] <= 1e-3, worst
    # Free-running, the FP32 and FP64 trajectories part through the contact events; compliance gradients
    # (proportional to constraint residuals of order 1e-5 m) feel that most.
    assert worst["free"] <= 1e-2, worst


def test_adjoint_contacts_vs_frozen_fd(jsb):
    """Through contact events: FP64 central FD whose perturbed runs replay the collision decisions of the
    GPU's run (planes in world space, contacts, friction clamps, restitution, velocity clamp), i.e. the
    derivative the adjoint computes with the collision active set frozen: within 1e-3 for positions,
    velocities and forces, 5e-3 for compliances (they act through constraint residuals of order 1e-5 m,
    which the FP32 trajectory resolves to about 1e-3; along the GPU's own trajectory the FP64 autodiff test
    above holds them to 1e-3)."""
    scene_bytes = contact_scene(jsb)
    scene, _ = parse_scene(scene_bytes)
    rng = np.random.default_rng(11)
    seeds = {24: {b: rng.standard_normal((body.num_vertices, 3)) for b, body in enumerate(scene.bodies)}}
    grads = gpu_gradients(jsb, scene_bytes, seeds, 24, 8)
    fd = FD64(scene, seeds, 24)
    errs = sample_and_compare(fd, grads, [(0, "x0", 6), (0, "force", 3), (1, "v0", 6), (1, "volume", 6), (1, "force", 3)],
                              rng, frozen=True)
    for kind, body, e, fds, gps in errs:
        print(kind, body, "rel", e, "\n  fd ", fds, "\n  gpu", gps)
    bar = {"x0": 1e-3, "v0": 1e-3, "force": 1e-3, "volume": 5e-3, "edge": 5e-3}
    assert all(e <= bar[k] for k, _, e, _, _ in errs), [(k, b, e) for k, b, e, _, _ in errs]


def test_checkpoint_interval_does_not_change_gradients(jsb):
    scene_bytes = build_scene("diff_batch", n_cloth=2, n_cube=1, steps=12)
    scene, _ = parse_scene(scene_bytes)
    rng = np.random.default_rng(3)
    seeds = {12: {b: rng.standard_normal((body.num_vertices, 3)) for b, body in enumerate(scene.bodies)}}
    a = gpu_gradients(jsb, scene_bytes, seeds, 12, 1)
    b = gpu_gradients(jsb, scene_bytes, seeds, 12, 5)
    for ga, gb in zip(a, b):
        for k in ga:
            assert np.array_equal(ga[k], gb[k]), k


def test_torch_autograd_binding(jsb):
    """rollout() as a torch.autograd.Function: its gradient equals the C ABI's and follows FD."""
    import torch

    from joltphysics_gb300.autograd import Simulation, rollout

    scene_bytes = build_scene("diff_cloth", n=8, steps=10)
    scene, _ = parse_scene(scene_bytes)
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    sim = Simulation(ctx, checkpoint_every=4)
    from jsb_testlib import blob_arrays, blob_compliance

    x0n, v0n, _ = blob_arrays(scene.bodies[0].blob)
    ecn, _ = blob_compliance(scene.bodies[0].blob)
    x0 = torch.tensor(x0n, dtype=torch.float32, requires_grad=True)
    v0 = torch.tensor(v0n, dtype=torch.float32, requires_grad=True)
    ec = torch.tensor(ecn, dtype=torch.float32, requires_grad=True)
    force = torch.zeros((1, 3), dtype=torch.float32, requires_grad=True)
    rng = np.random.default_rng(5)
    target = torch.tensor(rng.standard_normal((2, x0n.shape[0], 3)) * 0.01, dtype=torch.float32)
    pos = rollout(sim, x0, v0, ec, force, (5, 10))
    base = torch.tensor(np.asarray(scene.bodies[0].position, np.float32))
    loss = ((pos - (base + torch.tensor(x0n, dtype=torch.float32)) - target) ** 2).mean()
    loss.backward()
    assert torch.isfinite(x0.grad).all() and torch.isfinite(ec.grad).all() and torch.isfinite(force.grad).all()
    # d loss / d pos is linear in pos: check v0 gradient components against FP64 finite differences
    g_pos = (2.0 / pos.numel()) * (pos - (base + torch.tensor(x0n, dtype=torch.float32)) - target).detach().numpy()
    seeds = {5: {0: g_pos[0]}, 10: {0: g_pos[1]}}
    fd = FD64(scene, seeds, 10)
    for idx in [(3, 1), (20, 0), (40, 2)]:
        f = fd.central(0, "v0", idx, 1e-6)
        assert abs(float(v0.grad[idx]) - f) <= 1e-3 * max(abs(f), 1e-6), (idx, float(v0.grad[idx]), f)
    ctx.close()


def test_bulk_seed_and_gradients_equal_per_body(jsb):
    """jsb_adjoint_seed_all / jsb_adjoint_gradients_all == the per-body calls, and the last checkpoint
    segment taped during the forward pass gives the same gradients as a recomputed one (a second
    backward pass recomputes every segment)."""
    scene_bytes = build_scene("diff_batch", n_cloth=3, n_cube=2, steps=10)
    scene, _ = parse_scene(scene_bytes)
    rng = np.random.default_rng(8)
    seeds = {10: {b: rng.standard_normal((body.num_vertices, 3)) for b, body in enumerate(scene.bodies)}}
    per_body = gpu_gradients(jsb, scene_bytes, seeds, 10, 4)
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    ctx.set_scene_step_forces()
    pos = ctx.body_positions()
    for b in range(len(scene.bodies)):
        assert np.array_equal(pos[b], ctx.read_body(b)[0])
    ctx.adjoint_begin(10, 4)
    ctx.adjoint_forward()
    ctx.adjoint_seed_all(10, np.concatenate([seeds[10][b] for b in range(len(scene.bodies))]).astype(np.float32))
    ctx.adjoint_backward()
    bulk = ctx.adjoint_gradients_all()
    ctx.adjoint_backward()
    again = ctx.adjoint_gradients_all()
    ctx.adjoint_end()
    off = 0
    for b, g in enumerate(per_body):
        n = scene.bodies[b].num_vertices
        for key in ("x0", "v0"):
            assert np.array_equal(bulk[key][off:off + n], g[key]), (b, key)
            assert np.array_equal(again[key][off:off + n], g[key]), (b, key)
        assert np.array_equal(bulk["force"][b], g["force"]) and np.array_equal(again["force"][b], g["force"])
        off += n


def test_step_walk_adjoint_equals_substep_walk(jsb):
    """Differentiable run along the whole-step schedule (default) against the per-substep walk: the
    reverse sweep applies the same per-vertex and per-constraint reverse operations in the same order on
    every vertex, so position and velocity gradients agree bit for bit; force and compliance gradients
    are sums taken in another order (per thread, per whole-step slot) and agree to 1e-5. A cloth (whole-
    step walk) and a pressurised cube (per-substep walk in both) on a floor, through contact."""
    scene_bytes = build_scene("diff_batch", n_cloth=2, n_cube=1, steps=30, seed=3)
    scene, _ = parse_scene(scene_bytes)
    rng = np.random.default_rng(5)
    seeds = {15: {}, 30: {}}
    for b, body in enumerate(scene.bodies):
        for st in seeds:
            seeds[st][b] = rng.standard_normal((body.num_vertices, 3))
    a = gpu_gradients(jsb, scene_bytes, seeds, 30, 10)
    b = gpu_gradients(jsb, scene_bytes, seeds, 30, 10, step_walk=False)
    for i, (ga, gb) in enumerate(zip(a, b)):
        for key in ("x0", "v0"):
            assert np.array_equal(ga[key], gb[key]), (i, key, np.abs(ga[key] - gb[key]).max())
        for key in ("force", "edge_compliance", "volume_compliance"):
            x, y = np.asarray(ga[key], np.float64), np.asarray(gb[key], np.float64)
            if y.size:
                assert np.linalg.norm(x - y) <= 1e-5 * max(np.linalg.norm(y), 1e-30), (i, key)


def test_runs_in_one_context_reuse_buffers(jsb):
    """jsb_adjoint_end keeps the run's device buffers for the context's next differentiable run: a run,
    then one of another length and checkpoint interval (buffers grow and shrink), then the first again
    from the same state give bit-identical gradients."""
    scene_bytes = build_scene("diff_batch", n_cloth=3, n_cube=2, steps=12)
    scene, _ = parse_scene(scene_bytes)
    rng = np.random.default_rng(21)
    n = sum(b.num_vertices for b in scene.bodies)
    seed = rng.standard_normal((n, 3)).astype(np.float32)
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    ctx.set_scene_step_forces()
    init = ctx.save_all()

    def run(steps, every):
        ctx.restore_all(init)
        ctx.adjoint_begin(steps, every)
        ctx.adjoint_forward()
        ctx.adjoint_seed_all(steps, seed)
        ctx.adjoint_backward()
        g = ctx.adjoint_gradients_all()
        ctx.adjoint_end()
        return g

    first = run(10, 4)
    run(12, 3)
    again = run(10, 4)
    for key in ("x0", "v0", "force"):
        assert np.array_equal(first[key], again[key]), key
    ctx.close()


def test_tethered_cloth_adjoint_is_deterministic(jsb):
    """Several LRA tethers of one dependency level share an anchor (a pinned corner); their terms of the
    anchor's adjoint are summed in a fixed order, so two differentiable runs of a tethered cloth (no
    bends) give bit-identical gradients, and the gradients follow FP64 finite differences."""
    scene_bytes = build_scene("large_cloth", n=12, steps=8, bends=0)
    scene, _ = parse_scene(scene_bytes)
    from jsb_testlib import blob_counts_py

    assert blob_counts_py(scene.bodies[0].blob)["lra"] > 0
    rng = np.random.default_rng(12)
    nv = scene.bodies[0].num_vertices
    seeds = {4: {0: rng.standard_normal((nv, 3))}, 8: {0: rng.standard_normal((nv, 3))}}
    a = gpu_gradients(jsb, scene_bytes, seeds, 8, 3)
    b = gpu_gradients(jsb, scene_bytes, seeds, 8, 3)
    for key in ("x0", "v0", "force", "edge_compliance"):
        assert np.array_equal(a[0][key], b[0][key]), key
    fd = FD64(scene, seeds, 8)
    errs = sample_and_compare(fd, a, [(0, "x0", 8), (0, "v0", 8)], rng)
    for kind, body, e, fds, gps in errs:
        print(kind, body, "rel", e)
    # (a tether is a one-sided constraint: its activation |d| > max distance makes the loss only piecewise
    # smooth, so the bar is looser than for edges alone)
    assert max(e for _, _, e, _, _ in errs) <= 5e-3, [(k, e) for k, _, e, _, _ in errs]
