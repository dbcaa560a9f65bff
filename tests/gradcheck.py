"""Gradient checks of the hand-written adjoint at the two differentiable configurations (test and
benchmark infrastructure: used by tests/test_gpu_gradients_full.py and by bench.py's CPU checks).

Differentiable cloth (64 x 64, 120 steps, checkpoint every 10): loss = mean squared distance of all
vertex positions at steps 60 and 120 to a target run whose edge compliances are multiplied by
LogNormal(0, 0.3); gradients with respect to every edge compliance and initial velocity. References:
the gradient of a plain FP64 re-implementation (tests/torch_ref.py) by autodiff along the GPU's own
trajectory, and FP64 central finite differences of the oracle (free running).
Differentiable batch (256 bodies, 90 steps, checkpoint every 15): loss = sum over bodies of |centre of
mass at the last step - target|^2; gradients with respect to every body's step force and initial
velocity. References: FP64 autodiff of single bodies along the GPU's own trajectory, and FP64 central
finite differences of each perturbed body alone with the base run's collision decisions replayed.
"""
from __future__ import annotations

import numpy as np

from jsb_testlib import blob_arrays, blob_bend_compliance, blob_compliance, parse_scene, record32, run64, single_body_scene


def rel(a, b) -> float:
    return float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) / max(np.linalg.norm(b), 1e-300))


# ---- differentiable cloth ----------------------------------------------------------------------------
def cloth_target(jsb, scene_bytes, steps, seed=1) -> dict:
    """Target world positions after `steps` of a run with every edge compliance times LogNormal(0, 0.3)."""
    scene, _ = parse_scene(scene_bytes)
    ec, _ = blob_compliance(scene.bodies[0].blob)
    rng = np.random.default_rng(seed)
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    ctx.set_compliance(0, edge=(ec * np.exp(0.3 * rng.standard_normal(ec.shape))).astype(np.float32))
    out, cur = {}, 0
    for s in steps:
        ctx.step_graph(s - cur, 1)
        cur = s
        pos, loc, _ = ctx.read_body(0)
        out[s] = loc.astype(np.float64) + pos.astype(np.float64)
    ctx.close()
    return out


def cloth_adjoint(jsb, scene_bytes, steps, every, targets, trajectory=None):
    """GPU adjoint of the MSE loss: (gradients, loss). Fills trajectory[step] = [(world, velocities)]."""
    scene, _ = parse_scene(scene_bytes)
    n = scene.bodies[0].num_vertices
    m = 3.0 * n * len(targets)
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    ctx.adjoint_begin(steps, every)
    world = {}
    for s in range(1, steps + 1):
        if trajectory is None and s not in targets:
            continue
        ctx.adjoint_forward(s)
        pos, loc, vel = ctx.read_body(0)
        w = loc.astype(np.float64) + pos.astype(np.float64)
        if trajectory is not None:
            trajectory[s] = [(w, vel.astype(np.float64))]
        if s in targets:
            world[s] = w
    ctx.adjoint_forward()
    loss = 0.0
    for s, t in targets.items():
        loss += float(((world[s] - t) ** 2).sum()) / m
        ctx.adjoint_seed(s, 0, (2.0 * (world[s] - t) / m).astype(np.float32))
    ctx.adjoint_backward()
    g = ctx.adjoint_gradients(0, num_edges=len(blob_compliance(scene.bodies[0].blob)[0]))
    g["bend_compliance"] = ctx.adjoint_bend_gradients(0, len(blob_bend_compliance(scene.bodies[0].blob)))
    ctx.adjoint_end()
    ctx.close()
    return g, loss


def cloth_pinned_reference(scene, targets, trajectory):
    """FP64 autodiff of the same loss, the state moved onto the GPU trajectory after every step:
    ({"edge", "v0"} gradients, loss)."""
    import torch

    from torch_ref import base_params, simulate

    params = base_params(scene)
    out = simulate(scene, params, max(targets), sorted(targets), trajectory)
    m = 3.0 * scene.bodies[0].num_vertices * len(targets)
    loss = sum(((out[s][0] - torch.tensor(t)) ** 2).sum() for s, t in targets.items()) / m
    loss.backward()
    bend = params[0]["bend"].grad
    return ({"edge": params[0]["edge"].grad.numpy(), "v0": params[0]["v0"].grad.numpy(),
             "bend": bend.numpy() if bend is not None else np.zeros(0)}, float(loss.detach()))


def cloth_params(scene, rng, count=32):
    """count random parameters: half edge compliances (index), half initial velocity components ((i, k))."""
    n = scene.bodies[0].num_vertices
    ne = len(blob_compliance(scene.bodies[0].blob)[0])
    out = [("edge", int(i)) for i in rng.choice(ne, count // 2, replace=False)]
    out += [("v0", (int(rng.integers(n)), int(rng.integers(3)))) for _ in range(count - count // 2)]
    return out


def cloth_fd(scene, targets, params, eps_rel=1e-6, eps_abs=1e-6) -> np.ndarray:
    """FP64 central differences of the MSE loss (eps relative for compliances, absolute for velocities)."""
    x0, v0, _ = blob_arrays(scene.bodies[0].blob)
    ec, _ = blob_compliance(scene.bodies[0].blob)
    m = 3.0 * scene.bodies[0].num_vertices * len(targets)
    steps = max(targets)

    def loss(edge=ec, v=v0):
        out = run64(scene, 0, steps, set(targets), edge=edge, v0=v)
        return sum(float(((out[s] - t) ** 2).sum()) for s, t in targets.items()) / m

    fd = []
    for kind, idx in params:
        if kind == "edge":
            eps = eps_rel * ec[idx]
            a, b = ec.copy(), ec.copy()
            a[idx] += eps
            b[idx] -= eps
            fd.append((loss(edge=a) - loss(edge=b)) / (2 * eps))
        else:
            a, b = v0.copy(), v0.copy()
            a[idx] += eps_abs
            b[idx] -= eps_abs
            fd.append((loss(v=a) - loss(v=b)) / (2 * eps_abs))
    return np.array(fd)


def pick(g, params) -> tuple[np.ndarray, np.ndarray]:
    """GPU gradient components of `params`, split into (edge compliance, initial velocity)."""
    e = np.array([g["edge_compliance"][i] for k, i in params if k == "edge"], np.float64)
    v = np.array([g["v0"][i] for k, i in params if k == "v0"], np.float64)
    return e, v


def diff_cloth_check(jsb, build_scene, steps=120, every=10, loss_steps=(60, 120), fd_params=32, pinned=True, bends=False,
                     wave_mm=0) -> dict:
    """Relative errors of the GPU gradients: against FP64 autodiff along the GPU trajectory (pinned) and
    against free-running FP64 central differences on `fd_params` random parameters. bends: the same
    cloth with dihedral bends (then also d loss / d bend compliance against the pinned autodiff);
    wave_mm: the cloth starts as a height field of that amplitude instead of flat."""
    scene_bytes = build_scene("diff_cloth", steps=steps, bends=int(bends), wave_mm=int(wave_mm))
    scene, _ = parse_scene(scene_bytes)
    targets = cloth_target(jsb, scene_bytes, loss_steps)
    traj = {} if pinned else None
    g, loss = cloth_adjoint(jsb, scene_bytes, steps, every, targets, trajectory=traj)
    out = {"steps": steps, "loss_steps": list(loss_steps), "loss": loss}
    if pinned:
        ref, ref_loss = cloth_pinned_reference(scene, targets, traj)
        out["pinned_fp64_autodiff"] = {"edge_compliance": rel(g["edge_compliance"], ref["edge"]), "v0": rel(g["v0"], ref["v0"]),
                                       "loss_rel": abs(ref_loss - loss) / abs(loss)}
        if bends:
            out["pinned_fp64_autodiff"]["bend_compliance"] = rel(g["bend_compliance"], ref["bend"])
    if fd_params:
        params = cloth_params(scene, np.random.default_rng(4))
        fd = cloth_fd(scene, targets, params)
        ge, gv = pick(g, params)
        fe = np.array([f for (k, _), f in zip(params, fd) if k == "edge"])
        fv = np.array([f for (k, _), f in zip(params, fd) if k == "v0"])
        out["fp64_fd"] = {"parameters": len(params), "edge_compliance": rel(ge, fe), "v0": rel(gv, fv)}
    return out


# ---- differentiable batch ----------------------------------------------------------------------------
def batch_gradients(jsb, scene_bytes, steps=90, every=15, seed=17, trajectory_bodies=()):
    """GPU adjoint of the centre-of-mass loss: (force gradients (B, 3), per-body v0 gradients (B, 3),
    targets (B, 3), trajectory). trajectory[step] = {b: (world positions, velocities)} for the bodies in
    trajectory_bodies after every step."""
    scene, _ = parse_scene(scene_bytes)
    nb = len(scene.bodies)
    rng = np.random.default_rng(seed)
    targets = rng.normal(0.0, 1.0, (nb, 3)) + np.array([0.0, 0.5, 0.0])
    ctx = jsb.Context(0)
    ctx.load_scene(scene_bytes)
    ctx.set_scene_step_forces()
    counts = np.asarray(ctx.num_vertices, np.int64)
    offsets = np.concatenate([[0], np.cumsum(counts)])
    ctx.adjoint_begin(steps, every)
    trajectory = {}
    if trajectory_bodies:
        for s in range(1, steps + 1):
            ctx.adjoint_forward(s)
            trajectory[s] = {}
            for b in trajectory_bodies:
                pos, loc, vel = ctx.read_body(b)
                trajectory[s][b] = (loc.astype(np.float64) + pos.astype(np.float64), vel.astype(np.float64))
    ctx.adjoint_forward()
    loc = np.zeros((int(offsets[-1]), 3), np.float32)
    vel = np.zeros_like(loc)
    ctx.download_all(loc, vel)
    ctx.synchronize()
    com = np.add.reduceat(loc.astype(np.float64), offsets[:-1], axis=0) / counts[:, None] + ctx.body_positions()
    seed_dx = np.repeat(2.0 * (com - targets) / counts[:, None], counts, axis=0)
    ctx.adjoint_seed_all(steps, seed_dx.astype(np.float32))
    ctx.adjoint_backward()
    grads = ctx.adjoint_gradients_all()
    ctx.adjoint_end()
    ctx.close()
    # every vertex of a body starts with the body's v0: its gradient is the sum over the vertices
    return (grads["force"].astype(np.float64), np.add.reduceat(grads["v0"].astype(np.float64), offsets[:-1], axis=0), targets,
            trajectory)


def batch_pinned_reference(scene, b, target, steps, trajectory):
    """FP64 autodiff of body b's loss term, its state moved onto the GPU trajectory after every step:
    (force gradient (3,), v0 gradient summed over the vertices (3,))."""
    import torch

    from torch_ref import base_params, simulate

    sc = single_body_scene(scene, b)
    params = base_params(sc)
    pin = {s: [trajectory[s][b]] for s in trajectory}
    out = simulate(sc, params, steps, [steps], pin)
    loss = ((out[steps][0].mean(0) - torch.tensor(target, dtype=torch.float64)) ** 2).sum()
    loss.backward()
    return params[0]["force"].grad.numpy().copy(), params[0]["v0"].grad.numpy().sum(axis=0)


def pinned_bodies(scene, count_cloth=2, count_cube=1) -> list[int]:
    """The smallest cloths (no volume constraints) and tetrahedral cubes of a batch, by vertex count."""
    from jsb_testlib import blob_counts_py

    rows = [(scene.bodies[b].num_vertices, b, blob_counts_py(scene.bodies[b].blob)["volumes"] > 0) for b in range(len(scene.bodies))]
    cloths = [b for _, b, cube in sorted(rows) if not cube][:count_cloth]
    cubes = [b for _, b, cube in sorted(rows) if cube][:count_cube]
    return cloths + cubes


# central-difference steps: the step force enters as force * dt / vertices per substep, so its loss
# differences at 1e-6 N sit near the FP64 rounding noise of the run
FD_EPS = {"force": 1e-3, "v0": 1e-6}
# conditioning probe: relative size of the fixed perturbation of the FP64 state after every step, about the
# rounding the FP32 trajectory accumulates per step
PROBE_NOISE = 1e-6


def batch_fd(scene, b, kind, k, target, steps, eps=None, decisions=None, noise=0.0) -> float:
    """FP64 central difference of body b's loss term in its force or initial-velocity component k, the
    perturbed runs replaying `decisions` (an oracle with recorded collision decisions, by default those of
    the body's float run: the GPU's decisions, with planes, contacts, friction clamps, restitution and
    velocity clamp frozen as the adjoint has them). noise: see run64."""
    eps = FD_EPS[kind] if eps is None else eps
    body = scene.bodies[b]
    f0 = np.asarray(body.force, np.float64)
    _, v0, _ = blob_arrays(body.blob)
    replay = record32(scene, b, steps) if decisions is None else decisions
    vals = []
    for sgn in (1.0, -1.0):
        if kind == "force":
            f = f0.copy()
            f[k] += sgn * eps
            out = run64(scene, b, steps, {steps}, force=f, replay=replay, noise=noise)
        else:
            v = v0.copy()
            v[:, k] += sgn * eps
            out = run64(scene, b, steps, {steps}, v0=v, replay=replay, noise=noise)
        vals.append(float(((out[steps].mean(axis=0) - target) ** 2).sum()))
    return (vals[0] - vals[1]) / (2 * eps)


def diff_batch_check(jsb, build_scene, n_params=32, steps=90, every=15, pinned_counts=(2, 1)) -> dict:
    """GPU gradients against (pinned) FP64 autodiff of the smallest cloths and cubes (pinned_counts)
    along the GPU trajectory, and against FP64 central FD (replaying the collision decisions of the GPU's
    run, the derivative the adjoint computes) on n_params random (body, axis) parameters of distinct
    bodies, half force, half v0. A parameter is conditioned when its FD moves by at most 1e-4 (relative)
    under a fixed relative perturbation of PROBE_NOISE of the state after every step; for the others (the
    hanging cloths, which swing chaotically) the gradient is not determined to 1e-3 by any trajectory an
    FP32 solver computes, and only the pinned check applies."""
    scene_bytes = build_scene("diff_batch", steps=steps)
    scene, _ = parse_scene(scene_bytes)
    pin_bodies = pinned_bodies(scene, *pinned_counts)
    g_force, g_v0, targets, traj = batch_gradients(jsb, scene_bytes, steps, every, trajectory_bodies=pin_bodies)
    out = {"finite": bool(np.isfinite(g_force).all() and np.isfinite(g_v0).all())}
    if pin_bodies:
        ref = [batch_pinned_reference(scene, b, targets[b], steps, traj) for b in pin_bodies]
        out["pinned_fp64_autodiff"] = {
            "bodies": pin_bodies,
            "force": rel(np.concatenate([g_force[b] for b in pin_bodies]), np.concatenate([r[0] for r in ref])),
            "v0": rel(np.concatenate([g_v0[b] for b in pin_bodies]), np.concatenate([r[1] for r in ref]))}
    if not n_params:
        return out
    rng = np.random.default_rng(23)
    nb = len(scene.bodies)
    bodies = [int(b) for b in rng.permutation(nb)[:n_params]]
    picks = [("force" if i < n_params // 2 else "v0", b, int(rng.integers(3))) for i, b in enumerate(bodies)]
    rows = []
    for kind, b, k in picks:
        dec = record32(scene, b, steps)
        f = batch_fd(scene, b, kind, k, targets[b], steps, decisions=dec)
        fn = batch_fd(scene, b, kind, k, targets[b], steps, decisions=dec, noise=PROBE_NOISE)
        conditioned = abs(fn - f) <= 1e-4 * max(abs(f), 1e-12)
        gpu = float(g_force[b, k] if kind == "force" else g_v0[b, k])
        rows.append({"kind": kind, "body": b, "axis": k, "gpu": gpu, "fd": f, "fd_probe": fn, "conditioned": bool(conditioned)})
    out["parameters"] = len(rows)
    for kind in ("force", "v0"):
        sel = [r for r in rows if r["kind"] == kind and r["conditioned"]]
        out[kind] = {"conditioned": len(sel), "of": sum(r["kind"] == kind for r in rows),
                     "rel_error": rel([r["gpu"] for r in sel], [r["fd"] for r in sel]) if sel else None}
    ill = [r for r in rows if not r["conditioned"]]
    out["ill_conditioned_rel_error"] = rel([r["gpu"] for r in ill], [r["fd"] for r in ill]) if ill else None
    out["rows"] = rows
    return out
