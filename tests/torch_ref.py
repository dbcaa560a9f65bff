"""Plain FP64 re-implementation of the soft-body step in torch, for reference gradients by autodiff.

TEST INFRASTRUCTURE. It restates the same step as the CPU oracle (SoftBodyMotionProperties.cpp:
pressure :291-323, integration :325-365, dihedral bend :367-456 (through the signed angle, smooth at
flat triangle pairs), edge :573-601 / volume :458-507 / LRA :679-698 projections in
update-group order, collision + velocity update :700-825 against static boxes and spheres, velocity clamp
:827-921) in float64 with autograd. Collision planes are computed at the start of every step without
gradient (the collision active set is frozen, as in the GPU adjoint). Constraints are applied level by
level using the dependency levels of the library's schedule (each level touches disjoint written
vertices, so a vectorised level update equals the sequential order). The body is not recentered: world
positions are body position + local positions, which recentering leaves unchanged.
"""
from __future__ import annotations

import numpy as np
import torch

import joltphysics_gb300 as jsb
from jsb_testlib import Scene, blob_arrays, blob_bend_compliance, blob_compliance

F64 = torch.float64
PI32 = float(np.float32(np.pi))  # the reference's float constants (JPH_PI, Trigonometry.h)
ACOS_C = float(np.float32(0.175394))
FLT_MAX = 3.402823466e38


def _faces(blob: bytes) -> np.ndarray:
    import struct

    n = struct.unpack_from("<I", blob, 0)[0]
    off = 4 + 28 * n
    nf = struct.unpack_from("<I", blob, off)[0]
    return np.frombuffer(blob, np.uint32, 4 * nf, off + 4).reshape(nf, 4)[:, :3].astype(np.int64)


class BodyModel:
    def __init__(self, scene: Scene, b: int):
        body = scene.bodies[b]
        self.blob = body.blob
        cr = body.creation
        self.n_it, self.damping, self.max_v = int(cr[0]), float(cr[1]), float(cr[2])
        self.restitution, self.friction, self.pressure = float(cr[3]), float(cr[4]), float(cr[5])
        self.gravity_factor, self.radius = float(cr[6]), float(cr[7])
        self.position = np.asarray(body.position, np.float64)
        x0, v0, w = blob_arrays(body.blob)
        self.w = torch.tensor(w.astype(np.float64), dtype=F64)
        self.nv = len(w)
        self.faces = torch.tensor(_faces(body.blob))
        levels, records, source = jsb.settings_schedule(body.blob)
        self.levels = []
        L = len(levels) - 2
        for l in range(L):
            s, eb, ev, ee = (int(v) for v in levels[l])
            e = int(levels[l + 1][0])
            groups = {}
            for name, a, z in (("bend", s, eb), ("volume", eb, ev), ("edge", ev, ee), ("lra", ee, e)):
                if z <= a:
                    continue
                r = records[a:z]
                idx = np.stack([r[:, 0] & 0xFFFF, r[:, 0] >> 16, r[:, 1] & 0xFFFF, r[:, 1] >> 16], 1).astype(np.int64)
                groups[name] = (torch.tensor(idx), torch.tensor((source[a:z] & 0x0FFFFFFF).astype(np.int64)),
                                torch.tensor(r[:, 2].view(np.float32).astype(np.float64), dtype=F64),
                                torch.tensor(r[:, 3].view(np.float32).astype(np.float64), dtype=F64))
            self.levels.append(groups)


def _cross(a, b):
    return torch.cross(a, b, dim=-1)


def _dot(a, b):
    return (a * b).sum(-1)


def _planes(scene: Scene, m: BodyModel, x, v, P, bounds, dt):
    """Collision plane (normal, constant), shape index, friction and restitution per vertex (no grad)."""
    with torch.no_grad():
        nv = m.nv
        best = torch.full((nv,), -FLT_MAX, dtype=F64)
        normal = torch.zeros((nv, 3), dtype=F64)
        const = torch.zeros(nv, dtype=F64)
        shape = torch.full((nv,), -1, dtype=torch.long)
        mu, rest = [], []
        lmin, lmax = bounds
        wmin, wmax = P + lmin - m.radius, P + lmax + m.radius
        s = 0
        for c in scene.colliders:
            if c.type not in (0, 1):
                raise NotImplementedError("the FP64 reference models box and sphere colliders only")
            cp = np.asarray(c.position, np.float64)
            ext = np.asarray(c.half_extent if c.type == 0 else (c.radius,) * 3, np.float64)
            if np.any(wmin > cp + ext) or np.any(wmax < cp - ext):
                continue
            t = torch.tensor(cp - P, dtype=F64)
            if c.type == 0:
                h = torch.tensor(np.asarray(c.half_extent, np.float64), dtype=F64)
                local = x - t
                clamped = torch.maximum(torch.minimum(local, h), -h)
                inside = (clamped == local).all(-1)
                delta = h - local.abs()
                idx = delta.argmin(-1)
                pen_in = delta.gather(1, idx[:, None])[:, 0]
                n_in = torch.zeros_like(x)
                n_in[torch.arange(nv), idx] = torch.where(local[torch.arange(nv), idx] < 0, -1.0, 1.0).to(F64)
                c_in = -_dot(n_in, n_in * h) - _dot(t, n_in)
                d_out = local - clamped
                dist = d_out.norm(dim=-1)
                n_out = d_out / torch.clamp(dist, min=1e-300)[:, None]
                c_out = -_dot(n_out, clamped) - _dot(t, n_out)
                pen = torch.where(inside, pen_in, -dist)
                nn = torch.where(inside[:, None], n_in, n_out)
                cc = torch.where(inside, c_in, c_out)
            else:
                delta = x - t
                dist = delta.norm(dim=-1)
                pen = c.radius - dist
                nn = torch.where((dist > 0)[:, None], delta / torch.clamp(dist, min=1e-300)[:, None],
                                 torch.tensor([0.0, 1.0, 0.0], dtype=F64))
                cc = -_dot(nn, t + c.radius * nn)
            upd = (pen > best) & (m.w > 0)
            best = torch.where(upd, pen, best)
            normal = torch.where(upd[:, None], nn, normal)
            const = torch.where(upd, cc, const)
            shape = torch.where(upd, torch.full_like(shape, s), shape)
            mu.append(float(np.sqrt(np.float64(m.friction) * c.friction)))
            rest.append(max(m.restitution, c.restitution))
            s += 1
        return normal, const, shape, torch.tensor(mu + [0.0], dtype=F64), torch.tensor(rest + [0.0], dtype=F64)


def _bend_angle_term(theta):
    """sign(theta) ACosApproximate(cos |theta|) (Jolt/Math/Trigonometry.h:48-65), written so that it is
    smooth in theta at flat triangle pairs: sqrt(1 - cos t) = sqrt(2) sin(t / 2) for |t| <= pi / 2,
    sqrt(1 + cos t) = sqrt(2) cos(t / 2) beyond."""
    cos_t = torch.cos(theta)
    r2 = np.sqrt(2.0)
    near = r2 * torch.sin(0.5 * theta) * (PI32 / 2 - ACOS_C * cos_t)
    far = torch.where(theta < 0, -1.0, 1.0).to(F64) * (PI32 - r2 * torch.cos(0.5 * theta) * (PI32 / 2 + ACOS_C * cos_t))
    return torch.where(cos_t >= 0, near, far)


def _project_levels(m: BodyModel, x, edge_c, vol_c, k, bend_c=None):
    w = m.w
    for groups in m.levels:
        if "bend" in groups:  # SoftBodyMotionProperties.cpp:367-456
            idx, src, _, angle = groups["bend"]
            c_ = bend_c[src]
            i0, i1, i2, i3 = idx.T
            x0, x1, x2, x3 = x[i0], x[i1], x[i2], x[i3]
            e = x1 - x0
            el = e.norm(dim=-1)
            x1x2, x1x3 = x2 - x1, x3 - x1
            n1, n2 = _cross(x2 - x0, x1x2), _cross(x1x3, x3 - x0)
            n1s, n2s = _dot(n1, n1), _dot(n2, n2)
            ok = (el >= 1e-6) & (n1s * n2s >= 1e-24)
            n1s_, n2s_, el_ = (torch.where(ok, v, torch.ones_like(v)) for v in (n1s, n2s, el))
            theta = torch.atan2(_dot(_cross(n2, n1), e) / el_, _dot(n1, n2))
            c = _bend_angle_term(theta) - angle
            c = torch.where(c > PI32, c - 2 * PI32, torch.where(c < -PI32, c + 2 * PI32, c))
            n1h, n2h = n1 / n1s_[:, None], n2 / n2s_[:, None]
            d0 = (_dot(x1x2, e)[:, None] * n1h + _dot(x1x3, e)[:, None] * n2h) / el_[:, None]
            d2, d3 = el_[:, None] * n1h, el_[:, None] * n2h
            d1 = -d0 - d2 - d3
            w0, w1, w2, w3 = w[i0], w[i1], w[i2], w[i3]
            denom = w0 * _dot(d0, d0) + w1 * _dot(d1, d1) + w2 * _dot(d2, d2) + w3 * _dot(d3, d3) + c_ * k
            ok = (ok & (denom >= 1e-12))[:, None]
            ml = c / torch.where(denom >= 1e-12, denom, torch.ones_like(denom))
            for ii, xi, wi, di in ((i0, x0, w0, d0), (i1, x1, w1, d1), (i2, x2, w2, d2), (i3, x3, w3, d3)):
                x = x.index_put((ii,), torch.where(ok, xi - (ml * wi)[:, None] * di, xi))
        if "volume" in groups:
            idx, src, v0, _ = groups["volume"]
            c_ = vol_c[src]
            i1, i2, i3, i4 = idx.T
            x1, x2, x3, x4 = x[i1], x[i2], x[i3], x[i4]
            a, b, c = x2 - x1, x3 - x1, x4 - x1
            C = _dot(_cross(a, b), c).abs() - v0
            d1, d2, d3, d4 = _cross(x4 - x2, x3 - x2), _cross(b, c), _cross(c, a), _cross(a, b)
            w1, w2, w3, w4 = w[i1], w[i2], w[i3], w[i4]
            denom = w1 * _dot(d1, d1) + w2 * _dot(d2, d2) + w3 * _dot(d3, d3) + w4 * _dot(d4, d4) + c_ * k
            ok = (denom >= 1e-12)[:, None]
            ml = C / torch.where(denom >= 1e-12, denom, torch.ones_like(denom))
            for ii, xi, wi, di in ((i1, x1, w1, d1), (i2, x2, w2, d2), (i3, x3, w3, d3), (i4, x4, w4, d4)):
                x = x.index_put((ii,), torch.where(ok, xi - (ml * wi)[:, None] * di, xi))
        if "edge" in groups:
            idx, src, rest, _ = groups["edge"]
            c_ = edge_c[src]
            i0, i1 = idx[:, 0], idx[:, 1]
            x0, x1 = x[i0], x[i1]
            d = x1 - x0
            L = d.norm(dim=-1)
            denom = L * (w[i0] + w[i1] + c_ * k)
            ok = (denom >= 1e-12)[:, None]
            corr = d * ((L - rest) / torch.where(denom >= 1e-12, denom, torch.ones_like(denom)))[:, None]
            x = x.index_put((i0,), torch.where(ok, x0 + w[i0][:, None] * corr, x0))
            x = x.index_put((i1,), torch.where(ok, x1 - w[i1][:, None] * corr, x1))
        if "lra" in groups:
            idx, src, md, _ = groups["lra"]
            i0, i1 = idx[:, 0], idx[:, 1]
            d = x[i1] - x[i0]
            dls = _dot(d, d)
            act = (dls > md * md)[:, None]
            x = x.index_put((i1,), torch.where(act, x[i0] + d * (md / dls.clamp(min=1e-300).sqrt())[:, None], x[i1]))
    return x


def simulate(scene: Scene, params: list[dict], steps: int, observe: list[int], pin: dict | None = None):
    """params[b]: tensors x0 (N,3), v0 (N,3), edge (E,), volume (V,), force (3,). Returns {step: [world (N,3)]}.

    pin[step][b] = (world positions, velocities) of another run after `step`: the state is moved onto it
    at the end of that step with a straight-through term (values from the pinned run, derivatives of this
    one), so the gradient is evaluated along that run's trajectory.
    """
    g = torch.tensor(scene.gravity, dtype=F64)
    dt = float(np.float32(scene.dt))
    models = [BodyModel(scene, b) for b in range(len(scene.bodies))]
    states = []
    for m, p in zip(models, params):
        x = p["x0"]
        states.append({"x": x, "v": p["v0"], "bmin": x.detach().min(0).values.numpy(), "bmax": x.detach().max(0).values.numpy(),
                       "pmin": x.detach().min(0).values.numpy(), "pmax": x.detach().max(0).values.numpy()})
    out = {}
    for step in range(1, steps + 1):
        for b, (m, p, st) in enumerate(zip(models, params, states)):
            x, v = st["x"], st["v"]
            w = m.w[:, None]
            dts = dt / m.n_it
            k = 1.0 / (dts * dts)
            gb = m.gravity_factor * g
            damp = max(0.0, 1.0 - m.damping * dts)
            bounds = (np.minimum(st["bmin"], st["pmin"]), np.maximum(st["bmax"], st["pmax"]))
            normal, const, shape, mu, rest = _planes(scene, m, x, v, m.position, bounds, dt)
            thr = -2.0 * float(gb.norm()) * dts
            for it in range(m.n_it):
                if m.pressure > 0 and len(m.faces):
                    f = m.faces
                    x1, x2, x3 = x[f[:, 0]], x[f[:, 1]], x[f[:, 2]]
                    six = _dot(_cross(x1, x2), x3).sum()
                    if float(six.detach()) > 0:
                        imp = (m.pressure * dts / six) * _cross(x2 - x1, x3 - x1)
                        acc = torch.zeros_like(v)
                        for c in range(3):
                            acc = acc.index_add(0, f[:, c], imp)
                        v = v + w * acc
                sub_imp = p["force"] * dts / max(m.nv, 1)
                v = torch.where(w > 0, (v + (gb * dts + sub_imp * w)) * damp, v)
                prev = x
                x = x + v * dts
                x = _project_levels(m, x, p["edge"], p["volume"], k, p.get("bend"))
                # collision and velocity update (w > 0)
                pv = v
                vn0 = (x - prev) / dts
                has = (shape >= 0) & (m.w > 0)
                pd = -(_dot(x, normal) + const) + m.radius
                contact = (has & (pd > 0))[:, None]
                xc = torch.where(contact, x + normal * pd[:, None], x)
                vn = normal * _dot(normal, vn0)[:, None]
                vt = vn0 - vn
                vtl = vt.norm(dim=-1)
                sidx = shape.clamp(min=0)
                fr = torch.minimum(mu[sidx] * pd / (vtl.clamp(min=1e-300) * dts), torch.ones_like(pd))
                v1 = torch.where((vtl > 0)[:, None], vn0 - vt * fr[:, None], vn0)
                v2 = v1 - vn
                pvn = _dot(pv, normal)
                v3 = torch.where((pvn < thr)[:, None], v2 - (rest[sidx] * pvn)[:, None] * normal, v2)
                vnew = torch.where(contact, v3, vn0)
                v = torch.where(w > 0, vnew, v)
                x = torch.where(w > 0, xc, x)
            vsq = _dot(v, v)
            v = torch.where((vsq > m.max_v ** 2)[:, None], v * (m.max_v ** 2 / vsq.clamp(min=1e-300)).sqrt()[:, None], v)
            if pin is not None and step in pin:
                wx, wv = pin[step][b]
                x = x + (torch.tensor(np.asarray(wx, np.float64) - m.position, dtype=F64) - x.detach())
                v = v + (torch.tensor(np.asarray(wv, np.float64), dtype=F64) - v.detach())
            xd, vd = x.detach().numpy(), v.detach().numpy()
            disp = 0.5 * m.n_it * (m.n_it + 1) * dts * dts * gb.numpy()
            pred = xd + vd * dt + disp
            st.update(x=x, v=v, bmin=xd.min(0), bmax=xd.max(0), pmin=pred.min(0), pmax=pred.max(0))
        if step in observe:
            out[step] = [st["x"] + torch.tensor(m.position, dtype=F64) for m, st in zip(models, states)]
    return out


def base_params(scene: Scene, requires_grad=True) -> list[dict]:
    ps = []
    for body in scene.bodies:
        x0, v0, _ = blob_arrays(body.blob)
        ec, vc = blob_compliance(body.blob)
        bc = blob_bend_compliance(body.blob)
        p = {"x0": torch.tensor(x0, dtype=F64), "v0": torch.tensor(v0, dtype=F64), "edge": torch.tensor(ec, dtype=F64),
             "volume": torch.tensor(vc, dtype=F64), "force": torch.tensor(np.asarray(body.force, np.float64), dtype=F64),
             "bend": torch.tensor(bc, dtype=F64)}
        for t in p.values():
            t.requires_grad_(requires_grad)
        ps.append(p)
    return ps


def reference_gradients(scene: Scene, seeds: dict, steps: int, pin: dict | None = None):
    """Gradients of sum seed . world positions (same functional as FD64) by FP64 autodiff."""
    params = base_params(scene)
    out = simulate(scene, params, steps, sorted(seeds), pin)
    loss = 0.0
    for step, per_body in seeds.items():
        for b, r in per_body.items():
            loss = loss + (out[step][b] * torch.tensor(np.asarray(r, np.float64), dtype=F64)).sum()
    loss.backward()
    return [{k: (t.grad.numpy() if t.grad is not None else np.zeros(t.shape)) for k, t in p.items()} for p in params], float(loss)
