// Adjoint (reverse-mode) of the soft-body solver step on sm_103a.
//
// One CTA reverses one body through one step, substeps in reverse:
//   velocity clamp of UpdateSoftBodyState (last substep only)
//   ApplyCollisionConstraintsAndUpdateVelocities (SoftBodyMotionProperties.cpp:700-825), with the
//     collision active set frozen: the plane, shape index and the contact / friction-clamp /
//     restitution branch decisions are those of the forward pass
//   the constraint levels in reverse order (dihedral bend :367-456, edge :573-601, tetra volume
//     :458-507, LRA :679-698)
//   IntegratePositions (:325-365), accumulating d loss / d force
//   ApplyPressure (:291-323)
// Recentering of the body (UpdateSoftBodyState :882-898) moves local positions and the body
// position by opposite amounts; world positions, and so the adjoint, pass through it unchanged.
//
// The forward values each reverse stage needs come from the tape written by the taped forward step
// (constraint inputs, substep states, collision planes). Constraints of one level write disjoint
// vertices, so their reverse projections also run concurrently between barriers; an LRA anchor is only
// read, and the adjoint contributions of several LRA constraints to one anchor are summed after the
// level in a fixed order (lra_anchor_sums).
// d loss / d compliance accumulates per schedule slot; a slot is reversed by the same thread in every
// substep, so the accumulation is race free and deterministic.
//
// A body that walked its whole-step schedule forward (no pressure) is reversed along that schedule:
// the last velocity update, then its levels last to first, where a vertex slot reverses the integration
// of the substep the vertex entered and the velocity update of the one it left, then substep 0's
// integration. The taped forward step records the same substep states either way.
//
// Dihedral bends are differentiated through their signed angle (bend_adjoint), which keeps the
// derivative bounded at flat triangle pairs.

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "common.cuh"
#include "device_types.h"

namespace jsb {
namespace {

__device__ __forceinline__ f3 vzero() { return mk(0.0f, 0.0f, 0.0f); }
__device__ __forceinline__ int adj_slot_type(uint4 lv, uint32_t s) {
    return s < lv.y ? 0 : (s < lv.z ? 1 : (s < lv.w ? 2 : 3));
}

// x0' = x0 + w0 c, x1' = x1 - w1 c, c = d phi, d = x1 - x0, phi = (1 - rest / |d|) / (w0 + w1 + alpha k)
__device__ __forceinline__ void edge_adjoint(float4 *lx, const float *sw, uint4 r, const float4 *tin, float inv_dt_sq,
                                             float *grad) {
    const uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16;
    const float w0 = sw[i0], w1 = sw[i1];
    const float rest = __uint_as_float(r.z), alpha = __uint_as_float(r.w);
    const f3 dl = xyz(tin[0]);
    const float L = len(dl);
    const float s = w0 + w1 + alpha * inv_dt_sq;
    if (L * s < 1.0e-12f) return;
    const float phi = (1.0f - rest / L) / s;
    const f3 l0 = xyz(lx[i0]), l1 = xyz(lx[i1]);
    const f3 lc = w0 * l0 - w1 * l1;
    const float dc = dot(dl, lc);
    const f3 ld = phi * lc + dl * (rest / (L * L * L * s) * dc);
    lx[i0] = with_w(l0 - ld, 0.0f);
    lx[i1] = with_w(l1 + ld, 0.0f);
    *grad += dc * (-phi / s) * inv_dt_sq;
}

// x_i' = x_i - ml w_i d_i, ml = (|T| - V0) / (sum w_i |d_i|^2 + alpha k), T = (a x b) . c with
// a = x2 - x1, b = x3 - x1, c = x4 - x1 and d1 = (c - a) x (b - a), d2 = b x c, d3 = c x a, d4 = a x b.
__device__ __forceinline__ void volume_adjoint(float4 *lx, const float *sw, uint4 r, const float4 *tin, float inv_dt_sq,
                                               float *grad) {
    const uint32_t i1 = r.x & 0xffff, i2 = r.x >> 16, i3 = r.y & 0xffff, i4 = r.y >> 16;
    const float w1 = sw[i1], w2 = sw[i2], w3 = sw[i3], w4 = sw[i4];
    const float v0 = __uint_as_float(r.z), alpha = __uint_as_float(r.w);
    const f3 a = xyz(tin[0]), b = xyz(tin[1]), c = xyz(tin[2]);
    const f3 d1 = cross(c - a, b - a), d2 = cross(b, c), d3 = cross(c, a), d4 = cross(a, b);
    const float T = dot(d4, c);
    const float C = fabsf(T) - v0;
    const float denom = w1 * len_sq(d1) + w2 * len_sq(d2) + w3 * len_sq(d3) + w4 * len_sq(d4) + alpha * inv_dt_sq;
    if (denom < 1.0e-12f) return;
    const float ml = C / denom;
    const f3 L1 = xyz(lx[i1]), L2 = xyz(lx[i2]), L3 = xyz(lx[i3]), L4 = xyz(lx[i4]);
    const float lml = -(w1 * dot(d1, L1) + w2 * dot(d2, L2) + w3 * dot(d3, L3) + w4 * dot(d4, L4));
    const float lC = lml / denom;
    const float ldenom = -ml / denom * lml;
    const f3 G1 = (-ml * w1) * L1 + (2.0f * w1 * ldenom) * d1;
    const f3 G2 = (-ml * w2) * L2 + (2.0f * w2 * ldenom) * d2;
    const f3 G3 = (-ml * w3) * L3 + (2.0f * w3 * ldenom) * d3;
    const f3 G4 = (-ml * w4) * L4 + (2.0f * w4 * ldenom) * d4;
    *grad += ldenom * inv_dt_sq;
    const float lT = (T >= 0.0f ? 1.0f : -1.0f) * lC;
    f3 la = lT * cross(b, c), lb = lT * cross(c, a), lcv = lT * d4;
    // d1 = u x v, u = c - a, v = b - a
    const f3 lu = cross(b - a, G1), lv = cross(G1, c - a);
    lcv = lcv + lu;
    lb = lb + lv;
    la = la - (lu + lv);
    lb = lb + cross(c, G2);  // d2 = b x c
    lcv = lcv + cross(G2, b);
    lcv = lcv + cross(a, G3);  // d3 = c x a
    la = la + cross(G3, c);
    la = la + cross(b, G4);  // d4 = a x b
    lb = lb + cross(G4, a);
    lx[i1] = with_w(L1 - ((la + lb) + lcv), 0.0f);
    lx[i2] = with_w(L2 + la, 0.0f);
    lx[i3] = with_w(L3 + lb, 0.0f);
    lx[i4] = with_w(L4 + lcv, 0.0f);
}

// Dihedral bend (:367-456). The reference's constraint gradients d_i are exactly the gradients of the
// signed dihedral angle theta = atan2(((n2 x n1) . e) / |e|, n1 . n2) (|theta| = acos(n1 . n2 / |n1||n2|),
// its sign the reference's `sign`), and C = F(theta) - initial angle with F(theta) = sign(theta)
// ACosApproximate(cos |theta|). F is smooth in theta, flat triangle pairs included (there
// ACosApproximate's own derivative is unbounded but cos' vanishes), with
//   F'(theta) = h p / sqrt(2) + 0.175394 s sin|theta|,
//   cos|theta| >= 0: s = sqrt(1 - cos), p = pi/2 - 0.175394 cos, h = cos(|theta| / 2) = sqrt((1 + cos) / 2)
//   cos|theta| <  0: s = sqrt(1 + cos), p = pi/2 + 0.175394 cos, h = sin(|theta| / 2) = sqrt((1 - cos) / 2).
// So dC/dx_i = F'(theta) d_i. The map x_i' = x_i - ml w_i d_i, ml = C / (sum w_j |d_j|^2 + alpha k), is
// reversed through ml, C, the denominator and the d_i themselves (d0 = (((x2 - x1) . e) n1 / |n1|^2 +
// ((x3 - x1) . e) n2 / |n2|^2) / |e|, d2 = |e| n1 / |n1|^2, d3 = |e| n2 / |n2|^2, d1 = -d0 - d2 - d3,
// n1 = (x2 - x0) x (x2 - x1), n2 = (x3 - x1) x (x3 - x0), e = x1 - x0). Where the forward skipped the
// projection (|e| < 1e-6, |n1|^2 |n2|^2 < 1e-24, denominator < 1e-12) the adjoint passes through.
// Taped inputs: x1 - x0, x2 - x0, x3 - x0.
__device__ __forceinline__ void bend_adjoint(float4 *lx, const float *sw, uint4 r, const float4 *tin, float inv_dt_sq, float *grad) {
    const uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16, i2 = r.y & 0xffff, i3 = r.y >> 16;
    const float w[4] = {sw[i0], sw[i1], sw[i2], sw[i3]};
    const float alpha = __uint_as_float(r.z), angle = __uint_as_float(r.w);
    const f3 x1 = xyz(tin[0]), x2 = xyz(tin[1]), x3 = xyz(tin[2]);  // x0 = 0
    const f3 e = x1;
    const float el = len(e);
    if (el < 1.0e-6f) return;
    const f3 x1x2 = x2 - x1, x1x3 = x3 - x1;
    const f3 n1 = cross(x2, x1x2), n2 = cross(x1x3, x3);
    const float n1s = len_sq(n1), n2s = len_sq(n2), n1n2 = n1s * n2s;
    if (n1n2 < 1.0e-24f) return;
    const float sgn = dot(cross(n2, n1), e) < 0.0f ? -1.0f : 1.0f;
    float d = dot(n1, n2) / sqrtf(n1n2);
    float c = sgn * acos_approximate(d) - angle;
    if (c > kPi)
        c -= 2.0f * kPi;
    else if (c < -kPi)
        c += 2.0f * kPi;
    const f3 n1h = n1 / n1s, n2h = n2 / n2s;
    const float A = dot(x1x2, e), B = dot(x1x3, e);
    const f3 u = A * n1h + B * n2h;
    f3 D[4];
    D[0] = u / el;
    D[2] = el * n1h;
    D[3] = el * n2h;
    D[1] = (neg(D[0]) - D[2]) - D[3];
    const float den = w[0] * len_sq(D[0]) + w[1] * len_sq(D[1]) + w[2] * len_sq(D[2]) + w[3] * len_sq(D[3]) + alpha * inv_dt_sq;
    if (den < 1.0e-12f) return;
    const float ml = c / den;
    const uint32_t idx[4] = {i0, i1, i2, i3};
    f3 L[4], xb[4], Db[4];
    float mlb = 0.0f;
    for (int i = 0; i < 4; ++i) {
        L[i] = xyz(lx[idx[i]]);
        xb[i] = L[i];
        mlb -= w[i] * dot(L[i], D[i]);
    }
    const float cb = mlb / den, denb = -mlb * ml / den;
    *grad += denb * inv_dt_sq;
    // dC/dtheta
    d = fminf(1.0f, fmaxf(-1.0f, d));
    const float sinphi = sqrtf(fmaxf(0.0f, 1.0f - d * d));
    float s, pp, h;
    if (d >= 0.0f) {
        s = sqrtf(1.0f - d);
        pp = kPi / 2 - 0.175394f * d;
        h = sqrtf(0.5f * (1.0f + d));
    } else {
        s = sqrtf(1.0f + d);
        pp = kPi / 2 + 0.175394f * d;
        h = sqrtf(0.5f * (1.0f - d));
    }
    const float thb = cb * (h * pp * 0.70710678f + 0.175394f * s * sinphi);
    for (int i = 0; i < 4; ++i) {
        Db[i] = (-ml * w[i]) * L[i] + (2.0f * w[i] * denb) * D[i];
        xb[i] = xb[i] + thb * D[i];
    }
    // through d1 = -d0 - d2 - d3, d2 = el n1h, d3 = el n2h, d0 = u / el
    Db[0] = Db[0] - Db[1];
    Db[2] = Db[2] - Db[1];
    Db[3] = Db[3] - Db[1];
    float elb = dot(Db[2], n1h) + dot(Db[3], n2h) - dot(Db[0], D[0]) / el;
    const f3 ub = Db[0] / el;
    const float Ab = dot(ub, n1h), Bb = dot(ub, n2h);
    const f3 n1hb = el * Db[2] + A * ub, n2hb = el * Db[3] + B * ub;
    f3 x1x2b = Ab * e, x1x3b = Bb * e;
    f3 eb = Ab * x1x2 + Bb * x1x3;
    // n_h = n / |n|^2
    const f3 n1b = n1hb / n1s + (2.0f * (-dot(n1hb, n1h) / n1s)) * n1;
    const f3 n2b = n2hb / n2s + (2.0f * (-dot(n2hb, n2h) / n2s)) * n2;
    eb = eb + (elb / el) * e;
    // n1 = (x2 - x0) x x1x2, n2 = x1x3 x (x3 - x0)
    const f3 Pb = cross(x1x2, n1b);
    x1x2b = x1x2b + cross(n1b, x2);
    x1x3b = x1x3b + cross(x3, n2b);
    const f3 Vb = cross(n2b, x1x3);
    xb[2] = xb[2] + Pb + x1x2b;
    xb[3] = xb[3] + Vb + x1x3b;
    xb[1] = xb[1] - x1x2b - x1x3b + eb;
    xb[0] = xb[0] - Pb - Vb - eb;
    for (int i = 0; i < 4; ++i) lx[idx[i]] = with_w(xb[i], 0.0f);
}

// x1' = x0 + d md / |d| when |d| > md (d = x1 - x0); the anchor x0 is only read. The anchor's term is
// left in `anchor_term` (the slot's unused second tape entry) and added by lra_anchor_sums after the
// level: several tethers of one level may share an anchor.
__device__ __forceinline__ void lra_adjoint(float4 *lx, uint4 r, const float4 *tin, float4 *anchor_term) {
    const uint32_t i1 = r.x >> 16;
    const float md = __uint_as_float(r.z);
    const f3 dl = xyz(tin[0]);
    const float dls = len_sq(dl);
    if (!(dls > md * md)) {
        *anchor_term = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float L = sqrtf(dls);
    const f3 l = xyz(lx[i1]);
    const f3 ldl = (md / L) * (l - dl * (dot(dl, l) / dls));
    *anchor_term = with_w(l - ldl, 0.0f);
    lx[i1] = with_w(ldl, 0.0f);
}

// After a level's reverse: adds the anchor terms of its LRA slots [first, end) (schedule slot indices)
// to the anchors' adjoints, each anchor's terms summed in slot order by the thread holding the first of
// them (the host orders a level's LRA slots by anchor), so the result does not depend on thread timing.
template <int T>
__device__ __forceinline__ void lra_anchor_sums(float4 *lx, const uint4 *__restrict__ rec, const float4 *cons, uint32_t first,
                                                uint32_t end) {
    for (uint32_t c = first + threadIdx.x; c < end; c += T) {
        const uint4 r = __ldg(rec + c);
        if (r.x == 0xffffffffu) continue;
        const uint32_t a = r.x & 0xffff;
        if (c > first) {
            const uint32_t p = __ldg(rec + c - 1).x;
            if (p != 0xffffffffu && (p & 0xffff) == a) continue;  // not the first tether of its anchor
        }
        f3 acc = xyz(lx[a]);
        for (uint32_t k = c; k < end; ++k) {
            const uint32_t rk = __ldg(rec + k).x;
            if (rk == 0xffffffffu || (rk & 0xffff) != a) break;
            acc = acc + xyz(cons[size_t(k) * 3 + 1]);
        }
        lx[a] = with_w(acc, 0.0f);
    }
}


struct AdjShared {
    uint32_t item;
    float red[32];
    float v6, lcoef;
};

template <int T>
__device__ __forceinline__ float block_sum(AdjShared &sh, float v) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    __syncthreads();
    if (lane == 0) sh.red[warp] = v;
    __syncthreads();
    float t = 0.0f;
    for (int w = 0; w < T / 32; ++w) t += sh.red[w];
    __syncthreads();
    return t;  // every thread
}

// ---- asynchronous copies (cp.async, 16 bytes per thread) -----------------------------------------
__device__ __forceinline__ void adj_cp_async16(void *smem_dst, const void *gmem_src) {
    const uint32_t dst = uint32_t(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void adj_cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// Waits until at most `pending` (0 .. 3) of this thread's newest copy groups are still in flight.
__device__ __forceinline__ void adj_cp_async_wait(uint32_t pending) {
    if (pending >= 3)
        asm volatile("cp.async.wait_group 3;\n" ::: "memory");
    else if (pending == 2)
        asm volatile("cp.async.wait_group 2;\n" ::: "memory");
    else if (pending == 1)
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    else
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Reverse of one substep's constraint levels on the position adjoints lx.
//
// Thread t reverses slots t, t + T, ... of every level. The record and taped inputs of its first `rpt`
// slots are streamed `depth` levels ahead (in reverse level order) into the thread's own slice of a
// shared-memory ring with cp.async; a thread reads only what it copied itself, so the ring needs no
// barrier. Ring layout: [(depth + 1) levels][rpt slots][record, 3 taped inputs][T threads] x 16 bytes.
template <int T>
__device__ __forceinline__ void reverse_levels(float4 *lx, const float *sw, const BodyDesc &d, float4 *cons, float *grad,
                                               float inv_dt_sq, uint4 *ring, uint32_t depth, uint32_t rpt) {
    const uint4 *__restrict__ levels = d.levels;
    const uint4 *__restrict__ rec = d.records;
    const int L = int(d.num_levels);
    const uint32_t tid = threadIdx.x;
    const uint32_t nring = depth + 1;
    auto slot = [&](uint32_t l, uint32_t k) { return ring + ((l % nring) * rpt + k) * 4 * T + tid; };
    auto stage = [&](int l) {
        const uint4 lv = __ldg(levels + l);
        const uint32_t n = __ldg(levels + l + 1).x - lv.x;
        uint32_t s = tid;
        for (uint32_t k = 0; k < rpt && s < n; ++k, s += T) {
            const uint32_t c = lv.x + s;
            uint4 *dst = slot(uint32_t(l), k);
            const float4 *src = cons + size_t(c) * 3;
            adj_cp_async16(dst, rec + c);
            adj_cp_async16(dst + T, src);
            if (adj_slot_type(lv, s) <= 1) {
                adj_cp_async16(dst + 2 * T, src + 1);
                adj_cp_async16(dst + 3 * T, src + 2);
            }
        }
    };
    if (depth > 0)
        for (uint32_t k = 0; k < depth; ++k) {
            if (L - 1 - int(k) >= 0) stage(L - 1 - int(k));
            adj_cp_async_commit();
        }
    for (int l = L - 1; l >= 0; --l) {
        if (depth > 0) {
            if (l - int(depth) >= 0) stage(l - int(depth));
            adj_cp_async_commit();
            adj_cp_async_wait(depth);  // this thread's copies of level l have landed
        }
        const uint4 lv = __ldg(levels + l);
        const uint32_t n = __ldg(levels + l + 1).x - lv.x;
        uint32_t k = 0;
        for (uint32_t s = tid; s < n; s += T, ++k) {
            const uint32_t c = lv.x + s;
            const int type = adj_slot_type(lv, s);
            uint4 r;
            float4 tin[3];
            if (depth > 0 && k < rpt) {
                const uint4 *src = slot(uint32_t(l), k);
                r = src[0];
                tin[0] = *reinterpret_cast<const float4 *>(src + T);
                if (type <= 1) {
                    tin[1] = *reinterpret_cast<const float4 *>(src + 2 * T);
                    tin[2] = *reinterpret_cast<const float4 *>(src + 3 * T);
                }
            } else {
                r = __ldg(rec + c);
                const float4 *src = cons + size_t(c) * 3;
                tin[0] = src[0];
                if (type <= 1) {
                    tin[1] = src[1];
                    tin[2] = src[2];
                }
            }
            if (r.x == 0xffffffffu) continue;
            if (type == 2)
                edge_adjoint(lx, sw, r, tin, inv_dt_sq, grad + c);
            else if (type == 0)
                bend_adjoint(lx, sw, r, tin, inv_dt_sq, grad + c);
            else if (type == 1)
                volume_adjoint(lx, sw, r, tin, inv_dt_sq, grad + c);
            else if (type == 3)
                lra_adjoint(lx, r, tin, cons + size_t(c) * 3 + 1);
        }
        __syncthreads();
        if (lv.w < n) {  // LRA slots [lv.w, n)
            lra_anchor_sums<T>(lx, rec, cons, lv.x + lv.w, lv.x + n);
            __syncthreads();
        }
    }
    if (depth > 0) adj_cp_async_wait(0);
}

// Everything the per-vertex reverse passes of one body and step need.
struct VertexAdj {
    float4 *lx, *lv, *lp;
    const float *sw;
    const float4 *tape;  // this step's substep states [substep][3][nv]
    const float4 *planes;
    const int32_t *shapes;
    const float2 *cols;
    uint32_t nv, n_it;
    float dt_sub, inv_dt, damp, restitution_threshold, max_sq, radius;
};

// Reverse of ApplyCollisionConstraintsAndUpdateVelocities (:700-825) of substep `it` for vertex i, with
// the velocity clamp of UpdateSoftBodyState after the last substep: maps the adjoints of the position
// and velocity after the update to those of the position after the constraints (lx), the velocity
// before the update (lv, through restitution only) and the position at substep start (lp).
__device__ __forceinline__ void velocity_adjoint(const VertexAdj &a, uint32_t i, uint32_t it) {
    const float4 *ts = a.tape + size_t(it) * 3 * a.nv;
    const uint32_t nv = a.nv;
    const bool last = it == a.n_it - 1;
    const float w = a.sw[i];
    if (!(w > 0.0f)) {  // kinematic: position and velocity pass through; prev unused
        a.lp[i] = make_float4(0, 0, 0, 0);
        if (last) {  // velocity clamp of UpdateSoftBodyState
            const f3 vk = xyz(ts[nv + i]), lk = xyz(a.lv[i]);
            const float vsq = len_sq(vk);
            if (vsq > a.max_sq) a.lv[i] = with_w(sqrtf(a.max_sq / vsq) * (lk - vk * (dot(vk, lk) / vsq)), 0.0f);
        }
        return;
    }
    const f3 xs = xyz(ts[i]), pv = xyz(ts[nv + i]), xc = xyz(ts[2 * nv + i]);
    const f3 lxf = xyz(a.lx[i]);
    f3 lv3 = xyz(a.lv[i]);
    const f3 v0 = (xc - xs) * a.inv_dt;
    const int shape = a.shapes[i];
    bool contact = false;
    f3 n = vzero();
    float pd = 0.0f;
    if (shape >= 0) {
        const float4 pl = a.planes[i];
        n = xyz(pl);
        pd = -(dot(xc, n) + pl.w) + a.radius;
        contact = pd > 0.0f;
    }
    f3 vn = vzero(), vt = vzero(), v3 = v0;
    float vtl = 0.0f, f = 0.0f, mu = 0.0f, e = 0.0f;
    bool unclamped = false, rest = false;
    if (contact) {
        mu = a.cols[shape].x;
        e = a.cols[shape].y;
        vn = n * dot(n, v0);
        vt = v0 - vn;
        vtl = len(vt);
        f3 v1 = v0;
        if (vtl > 0.0f) {
            const float fq = mu * pd / (vtl * a.dt_sub);
            unclamped = !(fq > 1.0f);
            f = unclamped ? fq : 1.0f;
            v1 = v0 - vt * f;
        }
        const f3 v2 = v1 - vn;
        const float pvn = dot(pv, n);
        rest = pvn < a.restitution_threshold;
        v3 = rest ? v2 - (e * pvn) * n : v2;
    }
    if (last) {  // velocity clamp of UpdateSoftBodyState
        const float vsq = len_sq(v3);
        if (vsq > a.max_sq) {
            const float sc = sqrtf(a.max_sq / vsq);
            lv3 = sc * (lv3 - v3 * (dot(v3, lv3) / vsq));
        }
    }
    f3 lxc, lpv = vzero(), lv0;
    if (!contact) {
        lv0 = lv3;
        lxc = lxf;
    } else {
        if (rest) lpv = n * (-e * dot(n, lv3));
        const f3 lv1 = lv3;
        f3 lvn = vzero() - lv3;
        lv0 = lv1;
        f3 lvt = vzero();
        float lpd = 0.0f;
        if (vtl > 0.0f) {
            lvt = (-f) * lv1;
            if (unclamped) {
                const float lf = -dot(vt, lv1);
                lpd += mu / (vtl * a.dt_sub) * lf;
                const float lvtl = -f / vtl * lf;
                lvt = lvt + vt * (lvtl / vtl);
            }
        }
        lv0 = lv0 + lvt;
        lvn = lvn - lvt;
        lv0 = lv0 + n * dot(n, lvn);
        lpd += dot(n, lxf);
        lxc = lxf - n * lpd;
    }
    a.lx[i] = with_w(lxc + lv0 * a.inv_dt, 0.0f);
    a.lv[i] = with_w(lpv, 0.0f);
    a.lp[i] = with_w(vzero() - lv0 * a.inv_dt, 0.0f);
}

// Reverse of IntegratePositions (:325-365) for vertex i: x' = x + v' dt, v' = (v + g dt + F dt w / N) damp.
// Accumulates d loss / d (sub-step impulse) into force_acc.
__device__ __forceinline__ void integrate_adjoint(const VertexAdj &a, uint32_t i, f3 &force_acc) {
    const float w = a.sw[i];
    const f3 lxp = xyz(a.lx[i]);
    const f3 lvp = xyz(a.lv[i]) + lxp * a.dt_sub;
    f3 lvs = lvp;
    if (w > 0.0f) {
        lvs = lvp * a.damp;
        force_acc = force_acc + lvp * (w * a.damp);
    }
    a.lx[i] = with_w(lxp + xyz(a.lp[i]), 0.0f);
    a.lv[i] = with_w(lvs, 0.0f);
}

// Reverse of a whole-step walk (bodies without pressure that walked their whole-step schedule): the
// levels last to first; a constraint slot is reversed as in reverse_levels, a vertex slot {i, k} runs
// the reverse of substep k's integration, then of substep k - 1's velocity update. The ring works as in
// reverse_levels. d loss / d compliance accumulates per whole-step slot (the host sums a constraint's
// slots over the substeps).
template <int T>
__device__ __forceinline__ void reverse_step_levels(const VertexAdj &a, const BodyDesc &d, float4 *cons, float *grad,
                                                    float inv_dt_sq, uint4 *ring, uint32_t depth, uint32_t rpt, f3 &force_acc) {
    const uint4 *__restrict__ levels = d.step_levels;
    const uint4 *__restrict__ rec = d.step_records;
    const int L = int(d.num_step_levels);
    const uint32_t tid = threadIdx.x;
    const uint32_t nring = depth + 1;
    auto slot = [&](uint32_t l, uint32_t k) { return ring + ((l % nring) * rpt + k) * 4 * T + tid; };
    auto stage = [&](int l) {
        const uint4 lv = __ldg(levels + l);
        uint32_t s = tid;
        for (uint32_t k = 0; k < rpt && s < lv.w; ++k, s += T) {
            const uint32_t c = lv.x + s;
            const int type = step_slot_type(lv, s);
            uint4 *dst = slot(uint32_t(l), k);
            adj_cp_async16(dst, rec + c);
            if (type == 4) continue;
            const float4 *src = cons + size_t(c) * 3;
            adj_cp_async16(dst + T, src);
            if (type <= 1) {
                adj_cp_async16(dst + 2 * T, src + 1);
                adj_cp_async16(dst + 3 * T, src + 2);
            }
        }
    };
    if (depth > 0)
        for (uint32_t k = 0; k < depth; ++k) {
            if (L - 1 - int(k) >= 0) stage(L - 1 - int(k));
            adj_cp_async_commit();
        }
    for (int l = L - 1; l >= 0; --l) {
        if (depth > 0) {
            if (l - int(depth) >= 0) stage(l - int(depth));
            adj_cp_async_commit();
            adj_cp_async_wait(depth);  // this thread's copies of level l have landed
        }
        const uint4 lv = __ldg(levels + l);
        uint32_t k = 0;
        for (uint32_t s = tid; s < lv.w; s += T, ++k) {
            const uint32_t c = lv.x + s;
            const int type = step_slot_type(lv, s);
            uint4 r;
            float4 tin[3];
            const bool staged = depth > 0 && k < rpt;
            if (staged) {
                const uint4 *src = slot(uint32_t(l), k);
                r = src[0];
                if (type != 4) {
                    tin[0] = *reinterpret_cast<const float4 *>(src + T);
                    if (type <= 1) {
                        tin[1] = *reinterpret_cast<const float4 *>(src + 2 * T);
                        tin[2] = *reinterpret_cast<const float4 *>(src + 3 * T);
                    }
                }
            } else {
                r = __ldg(rec + c);
                if (type != 4) {
                    const float4 *src = cons + size_t(c) * 3;
                    tin[0] = src[0];
                    if (type <= 1) {
                        tin[1] = src[1];
                        tin[2] = src[2];
                    }
                }
            }
            if (r.x == 0xffffffffu) continue;
            if (type == 4) {
                integrate_adjoint(a, r.x, force_acc);
                velocity_adjoint(a, r.x, r.y - 1);
            } else if (type == 2) {
                edge_adjoint(a.lx, a.sw, r, tin, inv_dt_sq, grad + c);
            } else if (type == 0) {
                bend_adjoint(a.lx, a.sw, r, tin, inv_dt_sq, grad + c);
            } else if (type == 1) {
                volume_adjoint(a.lx, a.sw, r, tin, inv_dt_sq, grad + c);
            } else if (type == 3) {
                lra_adjoint(a.lx, r, tin, cons + size_t(c) * 3 + 1);
            }
        }
        __syncthreads();
        if ((lv.z & 0xffffu) < (lv.z >> 16)) {  // LRA slots [edge end, LRA end)
            lra_anchor_sums<T>(a.lx, rec, cons, lv.x + (lv.z & 0xffffu), lv.x + (lv.z >> 16));
            __syncthreads();
        }
    }
    if (depth > 0) adj_cp_async_wait(0);
}

// Shared memory (dynamic), cap = the launch's largest vertex count:
//   lx[cap] position adjoints | lv[cap] velocity adjoints | lp[cap] previous-position adjoints, then
//   substep positions for the pressure adjoint | w[cap] inverse masses | per-face pressure scratch
template <int T>
__device__ void adjoint_body(const AdjParams &q, uint32_t b, float4 *smem, uint32_t cap, uint32_t cap_faces, AdjShared &sh) {
    const uint32_t tid = threadIdx.x;
    const BodyDesc d = q.bodies[b];
    const TapeDesc td = q.tape[b];
    const uint32_t nv = d.num_vertices, n_it = d.num_iterations;
    float4 *lx = smem, *lv = smem + cap, *lp = smem + 2 * cap;
    float *sw = reinterpret_cast<float *>(smem + 3 * cap);
    float4 *sface = smem + 3 * cap + (cap + 3) / 4;
    uint4 *ring = reinterpret_cast<uint4 *>(sface + cap_faces);
    float4 *gax = q.adj_x + d.vtx_offset, *gav = q.adj_v + d.vtx_offset;

    const float dt_sub = q.dt / float(n_it);
    const f3 g = d.gravity_factor * ld3(q.gravity);
    const float inv_dt_sq = 1.0f / (dt_sub * dt_sub);
    float damp = 1.0f - d.linear_damping * dt_sub;
    damp = damp < 0.0f ? 0.0f : damp;
    const float inv_dt = 1.0f / dt_sub;
    const float restitution_threshold = -2.0f * len(g) * dt_sub;
    const float max_sq = d.max_linear_velocity * d.max_linear_velocity;
    const bool has_pressure = d.pressure > 0.0f && d.num_faces > 0;
    const float4 *planes = td.plane + size_t(q.tape_step) * nv;
    const int32_t *shapes = td.shape + size_t(q.tape_step) * nv;
    const float2 *cols = td.cols + size_t(q.tape_step) * kMaxCollidingShapes;
    const float4 *ts0 = td.state + size_t(q.tape_step) * n_it * 3 * nv;

    for (uint32_t i = tid; i < nv; i += T) {
        lx[i] = gax[i];
        lv[i] = gav[i];
        sw[i] = ts0[i].w;
    }
    __syncthreads();

    VertexAdj va;
    va.lx = lx;
    va.lv = lv;
    va.lp = lp;
    va.sw = sw;
    va.tape = ts0;
    va.planes = planes;
    va.shapes = shapes;
    va.cols = cols;
    va.nv = nv;
    va.n_it = n_it;
    va.dt_sub = dt_sub;
    va.inv_dt = inv_dt;
    va.damp = damp;
    va.restitution_threshold = restitution_threshold;
    va.max_sq = max_sq;
    va.radius = d.vertex_radius;

    f3 force_acc = vzero();
    const bool step_walk = d.step_levels != nullptr && !has_pressure && td.step_slots > 0;
    if (step_walk) {
        // the whole step walked as one schedule: last velocity update, the levels reversed (with the
        // per-vertex passes between substeps), substep 0's integration
        for (uint32_t i = tid; i < nv; i += T) velocity_adjoint(va, i, n_it - 1);
        __syncthreads();
        reverse_step_levels<T>(va, d, td.cons + size_t(q.tape_step) * td.step_slots * 3, td.grad, inv_dt_sq, ring, q.ring_depth,
                               q.ring_rpt, force_acc);
        for (uint32_t i = tid; i < nv; i += T) integrate_adjoint(va, i, force_acc);
        __syncthreads();
    }
    for (int it = step_walk ? -1 : int(n_it) - 1; it >= 0; --it) {
        const float4 *ts = td.state + (size_t(q.tape_step) * n_it + it) * 3 * nv;
        // ---- collision and velocity update ----
        for (uint32_t i = tid; i < nv; i += T) velocity_adjoint(va, i, uint32_t(it));
        __syncthreads();
        // ---- constraint levels, reversed ----
        reverse_levels<T>(lx, sw, d, td.cons + (size_t(q.tape_step) * n_it + it) * size_t(td.slots) * 3, td.grad, inv_dt_sq, ring,
                          q.ring_depth, q.ring_rpt);
        // ---- integration: x' = x + v' dt, v' = (v + g dt + F dt w / N) damp ----
        for (uint32_t i = tid; i < nv; i += T) integrate_adjoint(va, i, force_acc);
        __syncthreads();
        // ---- pressure: v += w coef (x2 - x1) x (x3 - x1) per face, coef = p dt / V6 ----
        if (has_pressure) {
            for (uint32_t i = tid; i < nv; i += T) lp[i] = ts[i];
            __syncthreads();
            float part = 0.0f;
            for (uint32_t f = tid; f < d.num_faces; f += T) {
                const uint4 fc = __ldg(d.faces + f);
                part += dot(cross(xyz(lp[fc.x]), xyz(lp[fc.y])), xyz(lp[fc.z]));
            }
            const float v6 = block_sum<T>(sh, part);
            if (v6 > 0.0f) {
                const float coef = d.pressure * dt_sub / v6;
                float lpart = 0.0f;
                for (uint32_t f = tid; f < d.num_faces; f += T) {
                    const uint4 fc = __ldg(d.faces + f);
                    const f3 x1 = xyz(lp[fc.x]), x2 = xyz(lp[fc.y]), x3 = xyz(lp[fc.z]);
                    const f3 gf = (sw[fc.x] * xyz(lv[fc.x]) + sw[fc.y] * xyz(lv[fc.y])) + sw[fc.z] * xyz(lv[fc.z]);
                    lpart += dot(gf, cross(x2 - x1, x3 - x1));
                    sface[f] = with_w(gf, 0.0f);
                }
                const float lcoef = block_sum<T>(sh, lpart);
                const float lv6 = -coef / v6 * lcoef;
                for (uint32_t i = tid; i < nv; i += T) {
                    f3 acc = xyz(lx[i]);
                    for (uint32_t k = __ldg(d.vf_off + i), ke = __ldg(d.vf_off + i + 1); k < ke; ++k) {
                        const uint32_t f = __ldg(d.vf + k);
                        const uint4 fc = __ldg(d.faces + f);
                        const f3 x1 = xyz(lp[fc.x]), x2 = xyz(lp[fc.y]), x3 = xyz(lp[fc.z]);
                        const f3 G = coef * xyz(sface[f]);
                        const f3 dx2 = cross(x3 - x1, G), dx3 = cross(G, x2 - x1);
                        if (i == fc.x)
                            acc = acc - (dx2 + dx3) + lv6 * cross(x2, x3);
                        else if (i == fc.y)
                            acc = acc + dx2 + lv6 * cross(x3, x1);
                        else
                            acc = acc + dx3 + lv6 * cross(x1, x2);
                    }
                    lx[i] = with_w(acc, 0.0f);
                }
            }
            __syncthreads();
        }
    }
    // d loss / d force: v' gets sub_imp w with sub_imp = F dt / N
    const float fs = dt_sub / float(nv > 0 ? nv : 1);
    const float fx = block_sum<T>(sh, force_acc.x), fy = block_sum<T>(sh, force_acc.y), fz = block_sum<T>(sh, force_acc.z);
    if (tid == 0) {
        q.grad_force[3 * b + 0] += fx * fs;
        q.grad_force[3 * b + 1] += fy * fs;
        q.grad_force[3 * b + 2] += fz * fs;
    }
    for (uint32_t i = tid; i < nv; i += T) {
        gax[i] = lx[i];
        gav[i] = lv[i];
    }
    __syncthreads();
}

template <int T>
__global__ void __launch_bounds__(T) adjoint_kernel(AdjParams q, uint32_t cap, uint32_t cap_faces) {
    extern __shared__ float4 smem[];
    __shared__ AdjShared sh;
    for (;;) {
        if (threadIdx.x == 0) sh.item = atomicAdd(q.queue, 1u);
        __syncthreads();
        const uint32_t item = sh.item;
        __syncthreads();
        if (item >= q.num_work) return;
        adjoint_body<T>(q, q.work[item], smem, cap, cap_faces, sh);
    }
}

__global__ void add_kernel(float4 *__restrict__ dst, const float4 *__restrict__ src, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
        float4 a = dst[i], b = src[i];
        dst[i] = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
    }
}

}  // namespace

// Dynamic shared memory of the adjoint CTA of `threads` threads: 3 adjoint arrays + inverse masses +
// pressure scratch + the level ring of `depth` levels ahead with `rpt` slots per thread.
size_t adjoint_smem_bytes(uint32_t vertices, uint32_t faces, uint32_t depth, uint32_t rpt, int threads) {
    const size_t ring = depth > 0 ? size_t(depth + 1) * rpt * 4 * size_t(threads) * sizeof(uint4) : 0;
    return size_t(vertices) * sizeof(float4) * 3 + size_t((vertices + 3) / 4) * sizeof(float4) + size_t(faces) * sizeof(float4) +
           ring;
}

cudaError_t init_adjoint_kernels(int max_dynamic_smem) {
    cudaError_t e = cudaFuncSetAttribute(adjoint_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(adjoint_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem);
    return e;
}

// threads: 128 or 256
int adjoint_occupancy(size_t smem, int threads) {
    int n = 0;
    if (threads == 256)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, adjoint_kernel<256>, 256, smem);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, adjoint_kernel<128>, 128, smem);
    return n;
}

cudaError_t launch_adjoint(const AdjParams &q, uint32_t cap_vertices, uint32_t cap_faces, int grid, int threads, cudaStream_t stream) {
    const size_t smem = adjoint_smem_bytes(cap_vertices, cap_faces, q.ring_depth, q.ring_rpt, threads);
    if (threads == 256)
        adjoint_kernel<256><<<grid, 256, smem, stream>>>(q, cap_vertices, cap_faces);
    else
        adjoint_kernel<128><<<grid, 128, smem, stream>>>(q, cap_vertices, cap_faces);
    return cudaGetLastError();
}

cudaError_t launch_add(float4 *dst, const float4 *src, uint64_t n, int num_sms, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    uint64_t blocks = (n + 255) / 256, cap = uint64_t(num_sms) * 8;
    add_kernel<<<unsigned(blocks < cap ? blocks : cap), 256, 0, stream>>>(dst, src, n);
    return cudaGetLastError();
}

}  // namespace jsb
