"""Thin torch.autograd binding of the GPU solver's hand-written adjoint (jsb_adjoint_* in include/jsb.h).

`rollout(sim, x0, v0, edge_compliance, force, observe)` runs the batched GPU step for max(observe) steps
and returns the world-space vertex positions of every body after each observed step; its backward pass
calls the library's adjoint (checkpointed recomputation, collision active set frozen) to produce
d loss / d initial local positions, initial velocities, per-edge compliance and per-body step force.
All tensors are float32; the solver state itself lives in the library, not in torch.
"""
from __future__ import annotations

import numpy as np
import torch

from . import Context


class Simulation:
    """A context plus the per-body parameter layout used by `rollout`."""

    def __init__(self, ctx: Context, checkpoint_every: int = 10):
        self.ctx = ctx
        self.checkpoint_every = checkpoint_every
        self.nv = list(ctx.num_vertices)
        self.offsets = np.concatenate([[0], np.cumsum(self.nv)]).astype(np.int64)
        self.positions = [np.asarray(b["position"], np.float32) for b in ctx.bodies]
        self.num_edges = [int(b["num_edges"]) for b in ctx.bodies]
        self.edge_offsets = np.concatenate([[0], np.cumsum(self.num_edges)]).astype(np.int64)

    @property
    def total_vertices(self) -> int:
        return int(self.offsets[-1])


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, edge_compliance, force, sim: Simulation, observe: tuple):
        c = sim.ctx
        xs = x0.detach().cpu().numpy().astype(np.float32)
        vs = v0.detach().cpu().numpy().astype(np.float32)
        c.upload_all(np.ascontiguousarray(xs), np.ascontiguousarray(vs))
        ec = edge_compliance.detach().cpu().numpy().astype(np.float32)
        fs = force.detach().cpu().numpy().astype(np.float32)
        for b in range(len(sim.nv)):
            c.set_compliance(b, edge=ec[sim.edge_offsets[b]:sim.edge_offsets[b + 1]])
            c.set_step_force(b, fs[b])
        steps = max(observe)
        c.adjoint_begin(steps, sim.checkpoint_every)
        out = []
        for s in sorted(observe):
            c.adjoint_forward(s)
            frame = np.zeros((sim.total_vertices, 3), np.float32)
            for b in range(len(sim.nv)):
                pos, loc, _ = c.read_body(b)
                frame[sim.offsets[b]:sim.offsets[b + 1]] = loc + pos
            out.append(frame)
        ctx.sim = sim
        ctx.observe = tuple(sorted(observe))
        return torch.from_numpy(np.stack(out)).to(x0.device)

    @staticmethod
    def backward(ctx, grad_out):
        sim: Simulation = ctx.sim
        c = sim.ctx
        g = grad_out.detach().cpu().numpy().astype(np.float32)
        for k, s in enumerate(ctx.observe):
            for b in range(len(sim.nv)):
                c.adjoint_seed(s, b, g[k, sim.offsets[b]:sim.offsets[b + 1]])
        c.adjoint_backward()
        dx = np.zeros((sim.total_vertices, 3), np.float32)
        dv = np.zeros((sim.total_vertices, 3), np.float32)
        de = np.zeros(int(sim.edge_offsets[-1]), np.float32)
        df = np.zeros((len(sim.nv), 3), np.float32)
        for b in range(len(sim.nv)):
            r = c.adjoint_gradients(b, num_edges=sim.num_edges[b])
            dx[sim.offsets[b]:sim.offsets[b + 1]] = r["x0"]
            dv[sim.offsets[b]:sim.offsets[b + 1]] = r["v0"]
            de[sim.edge_offsets[b]:sim.edge_offsets[b + 1]] = r["edge_compliance"]
            df[b] = r["force"]
        c.adjoint_end()
        dev = grad_out.device
        return (torch.from_numpy(dx).to(dev), torch.from_numpy(dv).to(dev), torch.from_numpy(de).to(dev),
                torch.from_numpy(df).to(dev), None, None)


def rollout(sim: Simulation, x0, v0, edge_compliance, force, observe) -> torch.Tensor:
    """World positions (len(observe), total_vertices, 3) after each observed step (1-based)."""
    return _Rollout.apply(x0, v0, edge_compliance, force, sim, tuple(observe))
