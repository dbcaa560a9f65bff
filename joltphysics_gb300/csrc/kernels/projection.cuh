// Per-vertex and per-constraint device arithmetic of the soft-body step, shared by the one-CTA
// solver (solver.cu) and the thread-block-cluster solver (cluster.cu). Same float operation order
// rules as common.cuh.
//
// The constraint projections take the position store as a template parameter: a plain shared-memory
// pointer (one CTA holds the whole body) or a cluster view (the body is spread over the shared memory
// of the CTAs of a cluster); ldx / stx read and write one vertex through either.
#pragma once

#include <float.h>

#include "common.cuh"
#include "device_types.h"

namespace jsb {
namespace {

__device__ __forceinline__ float4 ldx(const float4 *sx, uint32_t i) { return sx[i]; }
__device__ __forceinline__ void stx(float4 *sx, uint32_t i, float4 v) { sx[i] = v; }

struct SCol {  // one colliding shape, relative to the soft body
    int32_t type;
    int32_t flags;  // kColRotated: transform in c / ic / it (host-determined shapes); kColDynamic
    float t[3];
    float h[3];
    float r;
    float friction;
    float restitution;
    float isc;           // mSoftBodyInvMassScale
    int32_t hull;        // convex hulls: index into StepParams::hulls
    float c[9];          // rotation columns
    float ic[9], it[3];  // inverse transform (Mat44::InversedRotationTranslation): rotation columns, translation
};
enum : int32_t { kColRotated = 1, kColDynamic = 2, kColSensor = 4 };

// NaN positions (a body that has blown up in the reference's own arithmetic) would send every division
// and square root of a projection down the IEEE routines' slow path. For a body holding NaN positions
// the walkers run the projections with kGuard set, which test their inputs once instead: with a NaN
// coordinate among them, the reference's bend, volume and edge projections write NaN to every
// coordinate of every vertex they move (no early exit can be taken on a NaN; a bend's e_len exit only
// while x0 and x1 are finite), and that is written directly, as the canonical NaN the GPU's arithmetic
// produces, so the result is the same with or without the guard.
__device__ __forceinline__ bool has_nan(f3 a) { return a.x != a.x || a.y != a.y || a.z != a.z; }
__device__ __forceinline__ float4 nan_w(float w) {
    const float q = __int_as_float(0x7fffffff);
    return make_float4(q, q, q, w);
}

// ---------------------------------------------------------------------------------------------
// Constraint projections (exact reference arithmetic)
// ---------------------------------------------------------------------------------------------
// Each projection is written once over a division / square-root policy (common.cuh): it runs with
// FastOps, and when an operand fell outside FastOps' range it runs again with IeeeOps. The `_impl`
// functions store nothing on the first run unless FastOps stayed in range, and return true when the
// projection has to be repeated with IeeeOps; with IeeeOps they always finish (return false).
template <bool kGuard, class Ops, class X>
__device__ __forceinline__ bool project_bend_impl(X sx, uint4 r, float inv_dt_sq, Ops &op) {  // :367-456
    uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16, i2 = r.y & 0xffff, i3 = r.y >> 16;
    float compliance = __uint_as_float(r.z), initial_angle = __uint_as_float(r.w);
    float4 p0 = ldx(sx, i0), p1 = ldx(sx, i1), p2 = ldx(sx, i2), p3 = ldx(sx, i3);
    f3 x0 = xyz(p0), x1 = xyz(p1), x2 = xyz(p2), x3 = xyz(p3);
    if (kGuard && (has_nan(x0) || has_nan(x1) || has_nan(x2) || has_nan(x3))) {
        // e_len < 1e-6 is the only exit that can still be taken: with x0 and x1 finite and close
        if (!has_nan(x0) && !has_nan(x1) && len(x1 - x0) < 1.0e-6f) return false;
        stx(sx, i0, nan_w(p0.w));
        stx(sx, i1, nan_w(p1.w));
        stx(sx, i2, nan_w(p2.w));
        stx(sx, i3, nan_w(p3.w));
        return false;
    }
    f3 e = x1 - x0;
    float e_len = len_op(op, e);
    if (e_len < 1.0e-6f) return !op.ok();
    f3 x1x2 = x2 - x1, x1x3 = x3 - x1;
    f3 n1 = cross(x2 - x0, x1x2);
    f3 n2 = cross(x1x3, x3 - x0);
    float n1_len_sq = len_sq(n1), n2_len_sq = len_sq(n2);
    float n1n2 = n1_len_sq * n2_len_sq;
    if (n1n2 < 1.0e-24f) return !op.ok();
    float sign = dot(cross(n2, n1), e) < 0.0f ? -1.0f : 1.0f;
    float d = op.div(dot(n1, n2), op.sqrt(n1n2));
    float c = sign * acos_approximate_op(op, d) - initial_angle;
    if (c > kPi)
        c -= 2.0f * kPi;
    else if (c < -kPi)
        c += 2.0f * kPi;
    n1 = op.div3(n1, n1_len_sq);
    n2 = op.div3(n2, n2_len_sq);
    f3 d0c = op.div3(dot(x1x2, e) * n1 + dot(x1x3, e) * n2, e_len);
    f3 d2c = e_len * n1;
    f3 d3c = e_len * n2;
    f3 d1c = (neg(d0c) - d2c) - d3c;
    float w0 = p0.w, w1 = p1.w, w2 = p2.w, w3 = p3.w;
    float denom = w0 * len_sq(d0c) + w1 * len_sq(d1c) + w2 * len_sq(d2c) + w3 * len_sq(d3c) + compliance * inv_dt_sq;
    if (denom < 1.0e-12f) return !op.ok();
    float ml = op.div(c, denom);
    if (!op.ok()) return true;
    stx(sx, i0, with_w(x0 - (ml * w0) * d0c, w0));
    stx(sx, i1, with_w(x1 - (ml * w1) * d1c, w1));
    stx(sx, i2, with_w(x2 - (ml * w2) * d2c, w2));
    stx(sx, i3, with_w(x3 - (ml * w3) * d3c, w3));
    return false;
}

// The bend of project_bend_impl with FastOps, computed without branches up to the store: every value is
// computed speculatively (FastOps have no slow path and cannot fault), so the independent chains (edge
// length, the two normals, the angle, the gradients) overlap instead of waiting at each exit test; the
// exits are then taken in the reference's order with the values they would have seen. Same operations
// on the same operands as project_bend_impl, so the same bits. Returns true when FastOps went out of
// range before the projection's outcome was decided (the caller repeats it with IeeeOps).
template <class X>
__device__ __forceinline__ bool project_bend_fast(X sx, uint4 r, float inv_dt_sq) {
    const uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16, i2 = r.y & 0xffff, i3 = r.y >> 16;
    const float compliance = __uint_as_float(r.z), initial_angle = __uint_as_float(r.w);
    const float4 p0 = ldx(sx, i0), p1 = ldx(sx, i1), p2 = ldx(sx, i2), p3 = ldx(sx, i3);
    const f3 x0 = xyz(p0), x1 = xyz(p1), x2 = xyz(p2), x3 = xyz(p3);
    FastOps op;
    const f3 e = x1 - x0;
    const float e_len = len_op(op, e);
    const bool ok_len = op.ok();
    const f3 x1x2 = x2 - x1, x1x3 = x3 - x1;
    f3 n1 = cross(x2 - x0, x1x2);
    f3 n2 = cross(x1x3, x3 - x0);
    const float n1_len_sq = len_sq(n1), n2_len_sq = len_sq(n2);
    const float n1n2 = n1_len_sq * n2_len_sq;
    const float sign = dot(cross(n2, n1), e) < 0.0f ? -1.0f : 1.0f;
    const float d = op.div(dot(n1, n2), op.sqrt(n1n2));
    float c = sign * acos_approximate_op(op, d) - initial_angle;
    c = c > kPi ? c - 2.0f * kPi : (c < -kPi ? c + 2.0f * kPi : c);
    n1 = op.div3(n1, n1_len_sq);
    n2 = op.div3(n2, n2_len_sq);
    const f3 d0c = op.div3(dot(x1x2, e) * n1 + dot(x1x3, e) * n2, e_len);
    const f3 d2c = e_len * n1;
    const f3 d3c = e_len * n2;
    const f3 d1c = (neg(d0c) - d2c) - d3c;
    const float w0 = p0.w, w1 = p1.w, w2 = p2.w, w3 = p3.w;
    const float denom = w0 * len_sq(d0c) + w1 * len_sq(d1c) + w2 * len_sq(d2c) + w3 * len_sq(d3c) + compliance * inv_dt_sq;
    const bool ok_denom = op.ok();
    const float ml = op.div(c, denom);
    if (!ok_len) return true;
    if (e_len < 1.0e-6f || n1n2 < 1.0e-24f) return false;
    if (!ok_denom) return true;
    if (denom < 1.0e-12f) return false;
    if (!op.ok()) return true;
    stx(sx, i0, with_w(x0 - (ml * w0) * d0c, w0));
    stx(sx, i1, with_w(x1 - (ml * w1) * d1c, w1));
    stx(sx, i2, with_w(x2 - (ml * w2) * d2c, w2));
    stx(sx, i3, with_w(x3 - (ml * w3) * d3c, w3));
    return false;
}

template <bool kGuard, class Ops, class X>
__device__ __forceinline__ bool project_volume_impl(X sx, uint4 r, float inv_dt_sq, Ops &op) {  // :458-507
    uint32_t i1 = r.x & 0xffff, i2 = r.x >> 16, i3 = r.y & 0xffff, i4 = r.y >> 16;
    float six_rest = __uint_as_float(r.z), compliance = __uint_as_float(r.w);
    float4 p1 = ldx(sx, i1), p2 = ldx(sx, i2), p3 = ldx(sx, i3), p4 = ldx(sx, i4);
    f3 x1 = xyz(p1), x2 = xyz(p2), x3 = xyz(p3), x4 = xyz(p4);
    if (kGuard && (has_nan(x1) || has_nan(x2) || has_nan(x3) || has_nan(x4))) {
        stx(sx, i1, nan_w(p1.w));
        stx(sx, i2, nan_w(p2.w));
        stx(sx, i3, nan_w(p3.w));
        stx(sx, i4, nan_w(p4.w));
        return false;
    }
    f3 x1x2 = x2 - x1, x1x3 = x3 - x1, x1x4 = x4 - x1;
    float c = fabsf(dot(cross(x1x2, x1x3), x1x4)) - six_rest;
    f3 d1c = cross(x4 - x2, x3 - x2);
    f3 d2c = cross(x1x3, x1x4);
    f3 d3c = cross(x1x4, x1x2);
    f3 d4c = cross(x1x2, x1x3);
    float w1 = p1.w, w2 = p2.w, w3 = p3.w, w4 = p4.w;
    float denom = w1 * len_sq(d1c) + w2 * len_sq(d2c) + w3 * len_sq(d3c) + w4 * len_sq(d4c) + compliance * inv_dt_sq;
    if (denom < 1.0e-12f) return false;
    float ml = op.div(c, denom);
    if (!op.ok()) return true;
    stx(sx, i1, with_w(x1 - (ml * w1) * d1c, w1));
    stx(sx, i2, with_w(x2 - (ml * w2) * d2c, w2));
    stx(sx, i3, with_w(x3 - (ml * w3) * d3c, w3));
    stx(sx, i4, with_w(x4 - (ml * w4) * d4c, w4));
    return false;
}

template <bool kGuard, class Ops, class X>
__device__ __forceinline__ bool project_edge_impl(X sx, uint4 r, float inv_dt_sq, Ops &op) {  // :573-601
    uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16;
    float rest = __uint_as_float(r.z), compliance = __uint_as_float(r.w);
    float4 p0 = ldx(sx, i0), p1 = ldx(sx, i1);
    f3 x0 = xyz(p0), x1 = xyz(p1);
    if (kGuard && (has_nan(x0) || has_nan(x1))) {
        stx(sx, i0, nan_w(p0.w));
        stx(sx, i1, nan_w(p1.w));
        return false;
    }
    f3 delta = x1 - x0;
    float length = len_op(op, delta);
    float denom = length * (p0.w + p1.w + compliance * inv_dt_sq);
    if (denom < 1.0e-12f) return !op.ok();
    f3 corr = op.div3(delta * (length - rest), denom);
    if (!op.ok()) return true;
    stx(sx, i0, with_w(x0 + p0.w * corr, p0.w));
    stx(sx, i1, with_w(x1 - p1.w * corr, p1.w));
    return false;
}

// Edge and volume with FastOps, branch-free up to the store like project_bend_fast.
template <class X>
__device__ __forceinline__ bool project_edge_fast(X sx, uint4 r, float inv_dt_sq) {
    const uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16;
    const float rest = __uint_as_float(r.z), compliance = __uint_as_float(r.w);
    const float4 p0 = ldx(sx, i0), p1 = ldx(sx, i1);
    const f3 x0 = xyz(p0), x1 = xyz(p1);
    FastOps op;
    const f3 delta = x1 - x0;
    const float length = len_op(op, delta);
    const bool ok_len = op.ok();
    const float denom = length * (p0.w + p1.w + compliance * inv_dt_sq);
    const f3 corr = op.div3(delta * (length - rest), denom);
    if (!ok_len) return true;
    if (denom < 1.0e-12f) return false;
    if (!op.ok()) return true;
    stx(sx, i0, with_w(x0 + p0.w * corr, p0.w));
    stx(sx, i1, with_w(x1 - p1.w * corr, p1.w));
    return false;
}
template <class X>
__device__ __forceinline__ bool project_volume_fast(X sx, uint4 r, float inv_dt_sq) {
    const uint32_t i1 = r.x & 0xffff, i2 = r.x >> 16, i3 = r.y & 0xffff, i4 = r.y >> 16;
    const float six_rest = __uint_as_float(r.z), compliance = __uint_as_float(r.w);
    const float4 p1 = ldx(sx, i1), p2 = ldx(sx, i2), p3 = ldx(sx, i3), p4 = ldx(sx, i4);
    const f3 x1 = xyz(p1), x2 = xyz(p2), x3 = xyz(p3), x4 = xyz(p4);
    FastOps op;
    const f3 x1x2 = x2 - x1, x1x3 = x3 - x1, x1x4 = x4 - x1;
    const float c = fabsf(dot(cross(x1x2, x1x3), x1x4)) - six_rest;
    const f3 d1c = cross(x4 - x2, x3 - x2);
    const f3 d2c = cross(x1x3, x1x4);
    const f3 d3c = cross(x1x4, x1x2);
    const f3 d4c = cross(x1x2, x1x3);
    const float w1 = p1.w, w2 = p2.w, w3 = p3.w, w4 = p4.w;
    const float denom = w1 * len_sq(d1c) + w2 * len_sq(d2c) + w3 * len_sq(d3c) + w4 * len_sq(d4c) + compliance * inv_dt_sq;
    const float ml = op.div(c, denom);
    if (denom < 1.0e-12f) return false;
    if (!op.ok()) return true;
    stx(sx, i1, with_w(x1 - (ml * w1) * d1c, w1));
    stx(sx, i2, with_w(x2 - (ml * w2) * d2c, w2));
    stx(sx, i3, with_w(x3 - (ml * w3) * d3c, w3));
    stx(sx, i4, with_w(x4 - (ml * w4) * d4c, w4));
    return false;
}

template <class Ops, class X>
__device__ __forceinline__ bool project_lra_impl(X sx, uint4 r, Ops &op) {  // :679-698
    uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16;
    float md = __uint_as_float(r.z);
    f3 x0 = xyz(ldx(sx, i0));
    float4 p1 = ldx(sx, i1);
    f3 delta = xyz(p1) - x0;
    float dls = len_sq(delta);
    if (dls > md * md) {  // a NaN input fails the distance test: no division, no write
        f3 np = x0 + op.div3(delta * md, op.sqrt(dls));
        if (!op.ok()) return true;
        stx(sx, i1, with_w(np, p1.w));
    }
    return false;
}

template <bool kGuard = false, class X>
__device__ __forceinline__ void project_bend(X sx, uint4 r, float inv_dt_sq) {
    bool again;
    if (kGuard) {
        FastOps f;
        again = project_bend_impl<kGuard>(sx, r, inv_dt_sq, f);
    } else {
        again = project_bend_fast(sx, r, inv_dt_sq);
    }
    if (again) {
        IeeeOps e;
        project_bend_impl<kGuard>(sx, r, inv_dt_sq, e);
    }
}
template <bool kGuard = false, class X>
__device__ __forceinline__ void project_volume(X sx, uint4 r, float inv_dt_sq) {
    bool again;
    if (kGuard) {
        FastOps f;
        again = project_volume_impl<kGuard>(sx, r, inv_dt_sq, f);
    } else {
        again = project_volume_fast(sx, r, inv_dt_sq);
    }
    if (again) {
        IeeeOps e;
        project_volume_impl<kGuard>(sx, r, inv_dt_sq, e);
    }
}
template <bool kGuard = false, class X>
__device__ __forceinline__ void project_edge(X sx, uint4 r, float inv_dt_sq) {
    bool again;
    if (kGuard) {
        FastOps f;
        again = project_edge_impl<kGuard>(sx, r, inv_dt_sq, f);
    } else {
        again = project_edge_fast(sx, r, inv_dt_sq);
    }
    if (again) {
        IeeeOps e;
        project_edge_impl<kGuard>(sx, r, inv_dt_sq, e);
    }
}
template <class X>
__device__ __forceinline__ void project_lra(X sx, uint4 r) {
    FastOps f;
    if (project_lra_impl(sx, r, f)) {
        IeeeOps e;
        project_lra_impl(sx, r, e);
    }
}

// What a skinned constraint's projection reads besides the vertex: the body's constraint parameters and
// skin states, its switches and the substep (1-based iteration count mNextIteration / mNumIterations).
struct SkinRefs {
    const float4 *params;
    const float4 *state;
    float multiplier;
    uint32_t flags;
    uint32_t num_iterations;
    uint32_t substep;  // of a per-substep walk (whole-step records carry their own)
};

// ApplySkinConstraints (SoftBodyMotionProperties.cpp:509-571) for one constraint: the skinned position
// interpolated from the previous to the current skin state by the iteration, then the back stop sphere
// and the maximum distance, or the skinned position itself for a kinematic (max distance 0) vertex.
template <class X>
__device__ __forceinline__ void project_skin(X sx, uint4 r, const SkinRefs &sk, bool whole_step) {
    if (!(sk.flags & kSkinEnabled)) return;
    const uint32_t v = r.x & 0xffffu;
    const uint32_t substep = whole_step ? (r.x >> 16) : sk.substep;
    const float4 prm = sk.params[r.y & 0xffffffu];
    const float4 *st = sk.state + size_t(v) * 3;
    const float factor = (sk.flags & kSkinPreviousValid) ? div_rn(float(substep + 1), float(sk.num_iterations)) : 1.0f;
    const float prev_factor = 1.0f - factor;
    const float max_distance = prm.x * sk.multiplier;
    const f3 skin_pos = prev_factor * xyz(st[0]) + factor * xyz(st[1]);
    const float4 p = ldx(sx, v);
    f3 x = xyz(p);
    if (max_distance > 0.0f) {
        const float bsd = prm.y, bsr = prm.z;
        if (bsd < max_distance) {
            const f3 n = xyz(st[2]);
            const f3 center = skin_pos - n * (bsd + bsr);
            const f3 delta = x - center;
            const float dls = len_sq(delta);
            if (dls < bsr * bsr) {
                const float dl = sqrt_rn(dls);
                x = dl > 0.0f ? center + delta * div_rn(bsr, dl) : center + n * bsr;
            }
        }
        if (max_distance < FLT_MAX) {
            const f3 delta = x - skin_pos;
            const float dls = len_sq(delta);
            const float mds = max_distance * max_distance;
            if (dls > mds) x = skin_pos + delta * sqrt_rn(div_rn(mds, dls));
        }
    } else {
        x = skin_pos;
    }
    stx(sx, v, with_w(x, p.w));
}

template <bool kGuard = false, class X>
__device__ __forceinline__ void project(X sx, uint4 r, int type, float inv_dt_sq, const SkinRefs *sk = nullptr,
                                        bool whole_step = false) {
    if (type == 0)
        project_bend<kGuard>(sx, r, inv_dt_sq);
    else if (type == 1)
        project_volume<kGuard>(sx, r, inv_dt_sq);
    else if (type == 2) {
        if (r.y & 0x80000000u) {
            if (sk) project_skin(sx, r, *sk, whole_step);
        } else {
            project_edge<kGuard>(sx, r, inv_dt_sq);
        }
    } else
        project_lra(sx, r);
}

// Type of slot `s` of a level with descriptor {first slot, bend end, volume end, edge end}: the
// type groups are padded to multiples of 32 slots, so the type is uniform across a warp.
__device__ __forceinline__ int slot_type(uint4 lv, uint32_t s) {
    return s < lv.y ? 0 : (s < lv.z ? 1 : (s < lv.w ? 2 : 3));
}

// ---- asynchronous copies (cp.async, 16 bytes per thread) -----------------------------------------
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src) {
    const uint32_t dst = uint32_t(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---------------------------------------------------------------------------------------------
// Collision shapes
// ---------------------------------------------------------------------------------------------
// Plane::sFromPointAndNormal(point, normal).GetTransformed(translation t), identity rotation.
__device__ __forceinline__ float4 plane_transformed(f3 normal, f3 point, f3 t) {
    float c = -dot(normal, point);
    f3 n2;
    n2.x = (1.0f * normal.x + 0.0f * normal.y) + 0.0f * normal.z;
    n2.y = (0.0f * normal.x + 1.0f * normal.y) + 0.0f * normal.z;
    n2.z = (0.0f * normal.x + 0.0f * normal.y) + 1.0f * normal.z;
    return make_float4(n2.x, n2.y, n2.z, c - dot(t, n2));
}

// Mat44 * Vec3 with columns c0..c2 and translation t (Jolt/Math/Mat44.inl:295-302): ((c0 x + c1 y) + c2 z) + t.
__device__ __forceinline__ f3 mat_mul(const float *c, f3 v, f3 t) {
    return mk(((c[0] * v.x + c[3] * v.y) + c[6] * v.z) + t.x, ((c[1] * v.x + c[4] * v.y) + c[7] * v.z) + t.y,
              ((c[2] * v.x + c[5] * v.y) + c[8] * v.z) + t.z);
}
// Mat44::Multiply3x3 (Mat44.inl:384-390): (c0 x + c1 y) + c2 z.
__device__ __forceinline__ f3 mat_mul3(const float *c, f3 v) {
    return mk((c[0] * v.x + c[3] * v.y) + c[6] * v.z, (c[1] * v.x + c[4] * v.y) + c[7] * v.z, (c[2] * v.x + c[5] * v.y) + c[8] * v.z);
}

// Transform of a colliding shape relative to the soft body. XformT: a translation only (shapes the GPU
// finds among the context's colliders); XformR: a full rotation + translation (host-determined shapes),
// the shape's CollideSoftBodyVertices mapping the vertex with InversedRotationTranslation() and its
// plane back with Plane::GetTransformed (Jolt/Geometry/Plane.h:42-46).
struct XformT {
    f3 t;
    __device__ __forceinline__ f3 local(f3 p) const { return p + neg(t); }
    __device__ __forceinline__ float4 plane(f3 normal, f3 point) const { return plane_transformed(normal, point, t); }
};
struct XformR {
    const SCol &s;
    __device__ __forceinline__ f3 local(f3 p) const { return mat_mul(s.ic, p, ld3(s.it)); }
    __device__ __forceinline__ float4 plane(f3 normal, f3 point) const {
        const float c = -dot(normal, point);
        const f3 n2 = mat_mul3(s.c, normal);
        return make_float4(n2.x, n2.y, n2.z, c - dot(ld3(s.t), n2));
    }
};

// BoxShape::CollideSoftBodyVertices (BoxShape.cpp:234-283) for one vertex.
template <class X>
__device__ __forceinline__ void collide_box(f3 p, const SCol &s, const X &xf, int idx, float &largest, float4 &plane, int &shape) {
    f3 h = ld3(s.h);
    f3 local = xf.local(p);
    f3 clamped = vmax(vmin(local, h), neg(h));
    if (clamped.x == local.x && clamped.y == local.y && clamped.z == local.z) {
        f3 delta = h - mk(fabsf(local.x), fabsf(local.y), fabsf(local.z));
        int index = delta.x < delta.y ? (delta.z < delta.x ? 2 : 0) : (delta.z < delta.y ? 2 : 1);
        float pen = index == 0 ? delta.x : (index == 1 ? delta.y : delta.z);
        if (largest >= pen) return;
        largest = pen;
        f3 sgn = mk(signbit(local.x) ? -1.0f : 1.0f, signbit(local.y) ? -1.0f : 1.0f, signbit(local.z) ? -1.0f : 1.0f);
        f3 axis = mk(index == 0 ? 1.0f : 0.0f, index == 1 ? 1.0f : 0.0f, index == 2 ? 1.0f : 0.0f);
        f3 normal = mk(sgn.x * axis.x, sgn.y * axis.y, sgn.z * axis.z);
        f3 point = mk(normal.x * h.x, normal.y * h.y, normal.z * h.z);
        plane = xf.plane(normal, point);
        shape = idx;
    } else {
        f3 normal = local - clamped;
        float nl = len(normal);
        float pen = -nl;
        if (largest >= pen) return;
        largest = pen;
        normal = normal / nl;
        plane = xf.plane(normal, clamped);
        shape = idx;
    }
}

// SphereShape::CollideSoftBodyVertices (SphereShape.cpp:279-300) for one vertex (the centre is the
// transform's translation; the plane is already relative to the soft body).
__device__ __forceinline__ void collide_sphere(f3 p, const SCol &s, int idx, float &largest, float4 &plane, int &shape) {
    f3 center = ld3(s.t);
    f3 delta = p - center;
    float distance = len(delta);
    float pen = s.r - distance;
    if (largest >= pen) return;
    largest = pen;
    f3 normal = distance > 0.0f ? delta / distance : mk(0.0f, 1.0f, 0.0f);
    f3 point = center + s.r * normal;
    plane = make_float4(normal.x, normal.y, normal.z, -dot(normal, point));
    shape = idx;
}

// CapsuleShape::CollideSoftBodyVertices (CapsuleShape.cpp:324-374) for one vertex: a capsule along
// its Y axis, h[1] = half height of its cylinder part, r = radius.
template <class X>
__device__ __forceinline__ void collide_capsule(f3 p, const SCol &s, const X &xf, int idx, float &largest, float4 &plane, int &shape) {
    const float hh = s.h[1], r = s.r;
    const f3 local = xf.local(p);
    if (fabsf(local.y) <= hh) {  // beside the cylinder part: radial normal
        f3 normal = mk(local.x, 0.0f, local.z);
        const float nl = len(normal);
        const float pen = r - nl;
        if (largest >= pen) return;
        largest = pen;
        normal = nl > 0.0f ? normal / nl : mk(1.0f, 0.0f, 0.0f);
        plane = xf.plane(normal, r * normal);
    } else {  // beyond an end: the cap's sphere
        const f3 center = mk(0.0f, (local.y < 0.0f ? -1.0f : 1.0f) * hh, 0.0f);
        const f3 delta = local - center;
        const float distance = len(delta);
        const float pen = r - distance;
        if (largest >= pen) return;
        largest = pen;
        const f3 normal = delta / distance;
        plane = xf.plane(normal, center + r * normal);
    }
    shape = idx;
}

// Vec3::NormalizedOr (Jolt/Math/Vec3.inl:978-998, SSE4.1 form): v / |v|, or `zero` when
// |v|^2 = (x x + y y) + z z <= FLT_MIN.
__device__ __forceinline__ f3 normalized_or(f3 v, f3 zero) {
    const float px = v.x * v.x, py = v.y * v.y, pz = v.z * v.z;
    const float len_sq = (px + py) + pz;
    if (len_sq <= FLT_MIN) return zero;
    return v / jsqrt(len_sq);
}

// CylinderShape::CollideSoftBodyVertices (CylinderShape.cpp:317-368) for one vertex: a cylinder along its
// Y axis, h[1] = half height, r = radius. The plane is that of the closest surface (side, top / bottom,
// or the rim for a vertex outside both), its penetration measured from the plane.
template <class X>
__device__ __forceinline__ void collide_cylinder(f3 p, const SCol &s, const X &xf, int idx, float &largest, float4 &plane, int &shape) {
    const float hh = s.h[1], r = s.r;
    const f3 local = xf.local(p);
    const f3 side = mk(local.x, 0.0f, local.z);
    const float side_len = len(side);
    const float side_pen = r - side_len;
    const float top_pen = hh - fabsf(local.y);
    const float sgn = local.y < 0.0f ? -1.0f : 1.0f;
    f3 point, normal;
    if (side_pen < 0.0f && top_pen < 0.0f) {
        point = side * jdiv(r, side_len) + mk(0.0f, hh * sgn, 0.0f);
        normal = normalized_or(local - point, mk(0.0f, 1.0f, 0.0f));
    } else if (side_pen < top_pen) {
        normal = side_len > 0.0f ? side / side_len : mk(1.0f, 0.0f, 0.0f);
        point = r * normal;
    } else {
        normal = mk(0.0f, sgn, 0.0f);
        point = hh * normal;
    }
    const float c = -dot(normal, point);
    const float pen = -(dot(local, normal) + c);
    if (largest >= pen) return;
    largest = pen;
    plane = xf.plane(normal, point);
    shape = idx;
}

// ClosestPoint::GetClosestPointOnLine (Jolt/Geometry/ClosestPoint.h:15-43, 129-150): the point of segment
// (a, b) closest to the origin.
__device__ __forceinline__ f3 closest_point_on_line(f3 a, f3 b) {
    const f3 ab = b - a;
    const float den = len_sq(ab);
    float u, v;
    if (den < FLT_EPSILON * FLT_EPSILON) {
        const bool a_closer = len_sq(a) < len_sq(b);
        u = a_closer ? 1.0f : 0.0f;
        v = a_closer ? 0.0f : 1.0f;
    } else {
        v = jdiv(-dot(a, ab), den);
        u = 1.0f - v;
    }
    if (v <= 0.0f) return a;
    if (u <= 0.0f) return b;
    return u * a + v * b;
}

// Registered convex hulls (jsb_hull_add).
struct HullRefs {
    const HullDev *hulls;
    const float4 *f4;
    const uint32_t *u32;
};

// ConvexHullShape::CollideSoftBodyVertices (ConvexHullShape.cpp:1060-1163), unscaled, for one vertex: the
// most facing plane; outside the hull the closest point on that face's edges where the vertex lies
// beyond them; the plane through the closest point.
__device__ __forceinline__ void collide_hull(f3 p, const SCol &s, const XformR &xf, const HullRefs &hr, int idx, float &largest,
                                             float4 &plane, int &shape) {
    const HullDev h = hr.hulls[s.hull];
    const f3 local = xf.local(p);
    float max_distance = -FLT_MAX;
    f3 max_n = mk(0.0f, 0.0f, 0.0f);
    uint32_t max_i = 0;
    for (uint32_t i = 0; i < h.num_faces; ++i) {
        const float4 pl = hr.f4[h.f4 + i];
        const float distance = dot(local, xyz(pl)) + pl.w;
        if (distance > max_distance) {
            max_distance = distance;
            max_n = xyz(pl);
            max_i = i;
        }
    }
    f3 closest = (-max_distance) * max_n;
    const bool outside = max_distance > 0.0f;
    if (outside) {
        float best = FLT_MAX;
        const uint32_t first = hr.u32[h.faces + 2 * max_i], count = hr.u32[h.faces + 2 * max_i + 1];
        const float4 *points = hr.f4 + h.f4 + h.num_faces;
        for (uint32_t k = 0; k < count; ++k) {
            const f3 p1 = xyz(points[hr.u32[first + k]]);
            const f3 p2 = xyz(points[hr.u32[first + (k + 1 == count ? 0 : k + 1)]]);
            if (dot(cross(p2 - p1, max_n), local - p1) > 0.0f) {  // beyond this edge
                const f3 c = closest_point_on_line(p1 - local, p2 - local);
                const float dsq = len_sq(c);
                if (dsq < best) {
                    best = dsq;
                    closest = c;
                }
            }
        }
    }
    f3 normal = neg(closest);
    const float nl = len(normal);
    float pen = nl;
    if (outside)
        pen = -pen;
    else
        normal = neg(normal);
    if (largest >= pen) return;
    largest = pen;
    normal = nl > 1.0e-12f ? normal / nl : max_n;
    plane = xf.plane(normal, local + closest);
    shape = idx;
}

template <class X>
__device__ __forceinline__ void collide_shape(f3 x, const SCol &s, const X &xf, int idx, float &largest, float4 &plane, int &shape) {
    switch (s.type) {
        case 0: collide_box(x, s, xf, idx, largest, plane, shape); break;
        case 1: collide_sphere(x, s, idx, largest, plane, shape); break;
        case 2: collide_capsule(x, s, xf, idx, largest, plane, shape); break;
        default: collide_cylinder(x, s, xf, idx, largest, plane, shape); break;
    }
}

// ---------------------------------------------------------------------------------------------
// Reductions for UpdateSoftBodyState
// ---------------------------------------------------------------------------------------------
// Sequential AABox::Encapsulate keeps, among equal extreme values, the last vertex in index order
// (mMin = mMin < p ? mMin : p). Reducing (value, index) pairs with "strictly better, else larger
// index" reproduces that choice (it matters only for the sign of zero).
__device__ __forceinline__ void pick_min(float &v, int &i, float ov, int oi) {
    if (ov < v || (!(v < ov) && oi > i)) {
        v = ov;
        i = oi;
    }
}
__device__ __forceinline__ void pick_max(float &v, int &i, float ov, int oi) {
    if (ov > v || (!(v > ov) && oi > i)) {
        v = ov;
        i = oi;
    }
}

// DetermineCollisionPlanes (SoftBodyMotionProperties.cpp:257-265) for one vertex: the plane of the
// colliding shape with the largest penetration (strictly larger replaces, CollideSoftBodyVertexIterator.h:86).
// Returns the shape index, -1 for none.
__device__ __forceinline__ int collision_plane(f3 x, const SCol *cols, int ncols, float4 &plane, const HullRefs &hr = HullRefs{}) {
    int shape = -1;
    float largest = -FLT_MAX;
    for (int s = 0; s < ncols; ++s) {
        if (cols[s].flags & kColSensor) continue;  // (host-determined shapes only; sensor_hits)
        if (cols[s].type == 4)  // (host-determined shapes only)
            collide_hull(x, cols[s], XformR{cols[s]}, hr, s, largest, plane, shape);
        else if (cols[s].flags & kColRotated)
            collide_shape(x, cols[s], XformR{cols[s]}, s, largest, plane, shape);
        else
            collide_shape(x, cols[s], XformT{ld3(cols[s].t)}, s, largest, plane, shape);
    }
    return shape;
}

// DetermineSensorCollisions (:267-289) for one vertex (inverse mass > 0): bit s set for each sensor shape s
// the vertex penetrates. The reference shares one penetration over all vertices of a sensor and reports a
// contact when the largest is positive, that is when some vertex penetrates.
__device__ __forceinline__ uint32_t sensor_hits(f3 x, const SCol *cols, int ncols, uint32_t sensors, const HullRefs &hr) {
    uint32_t hits = 0;
    for (int s = 0; s < ncols; ++s) {
        if (!((sensors >> s) & 1u)) continue;
        float largest = -FLT_MAX;
        float4 plane;
        int shape = -1;
        if (cols[s].type == 4)
            collide_hull(x, cols[s], XformR{cols[s]}, hr, s, largest, plane, shape);
        else
            collide_shape(x, cols[s], XformR{cols[s]}, s, largest, plane, shape);
        if (largest > 0.0f) hits |= 1u << s;
    }
    return hits;
}

// ApplyCollisionConstraintsAndUpdateVelocities (:700-825), static-collider branch (:798-816), for one
// vertex with a collision plane: if it penetrates, pushes x out along the normal, applies friction,
// removes the normal velocity and adds restitution. v is the velocity (x - prev) / dt_sub, prev_v the
// velocity before the constraint projection. Returns whether the vertex was in contact.
__device__ __forceinline__ bool collide_vertex(f3 &x, f3 &v, f3 prev_v, float4 pl, const SCol &cs, float radius, float dt_sub,
                                               float restitution_threshold) {
    f3 n = xyz(pl);
    float projected = -(dot(x, n) + pl.w) + radius;
    if (!(projected > 0.0f)) return false;
    x = x + n * projected;
    if (!(cs.isc > 0.0f)) return true;  // the soft body is not moved by this shape (mSoftBodyInvMassScale = 0)
    f3 v_normal = n * dot(n, v);
    f3 v_tan = v - v_normal;
    float vtl = sqrt_rn(len_sq(v_tan));
    if (vtl > 0.0f) {
        float fr = div_rn(cs.friction * projected, vtl * dt_sub);
        fr = fr < 1.0f ? fr : 1.0f;  // min(fr, 1)
        v = v - v_tan * fr;
    }
    v = v - v_normal;
    float pvn = dot(prev_v, n);
    if (pvn < restitution_threshold) v = v - (cs.restitution * pvn) * n;
    return true;
}

// The dynamic-body branch of ApplyCollisionConstraintsAndUpdateVelocities (:752-797) for one vertex
// whose collision plane belongs to a dynamic shape: pushes x out of the plane, then exchanges an impulse
// between the vertex and the body (friction and restitution against the body's point velocity), updating
// the body's velocities lin / ang in place, which the next vertex in index order sees. Returns whether an
// impulse was applied (CollidingShape::mUpdateVelocities).
__device__ __forceinline__ bool collide_vertex_dynamic(f3 &x, f3 &v, f3 prev_v, float w, float4 pl, const ShapeEntry &e, f3 &lin,
                                                       f3 &ang, float radius, float dt_sub, float restitution_threshold, bool &contact) {
    const f3 n = xyz(pl);
    const float projected = -(dot(x, n) + pl.w) + radius;
    contact = projected > 0.0f;
    if (!contact) return false;
    x = x + n * projected;
    const f3 r2 = x - ld3(e.com);
    const f3 v2 = lin + cross(ang, r2);  // CollidingShape::GetPointVelocity
    const f3 relative = v - v2;
    const f3 v_normal = n * dot(n, relative);
    const f3 v_tan = relative - v_normal;
    const float vtl = sqrt_rn(len_sq(v_tan));
    const float vertex_inv_mass = e.inv_mass_scale * w;
    const f3 r2xn = cross(r2, n);
    const float w2 = e.inv_mass + dot(r2xn, mat_mul(e.inv_inertia, r2xn, ld3(e.inv_inertia + 9)));
    const float w12 = vertex_inv_mass + w2;
    if (!(w12 > 0.0f)) return false;
    f3 dv = mk(0.0f, 0.0f, 0.0f);
    if (vtl > 0.0f) {
        float fr = div_rn(e.friction * projected, vtl * dt_sub);
        fr = fr < 1.0f ? fr : 1.0f;
        dv = v_tan * fr;
    }
    dv = dv + v_normal;
    const float pvn = dot(prev_v - v2, n);
    if (pvn < restitution_threshold) dv = dv + (e.restitution * pvn) * n;
    const f3 imp = div3_rn(dv, w12);
    v = v - imp * vertex_inv_mass;
    lin = lin + imp * e.inv_mass;
    ang = ang + mat_mul(e.inv_inertia, cross(r2, imp), ld3(e.inv_inertia + 9));
    return true;
}

// DetermineCollidingShapes (SoftBodyMotionProperties.cpp:120-255) for static colliders: every shape whose
// world AABB overlaps the body's bounds U predicted bounds, grown by the vertex radius, with combined
// friction sqrt(f1 * f2) and restitution max(r1, r2) (ContactConstraintManager.h:554-555). Returns the count.
__device__ inline int colliding_shapes(const StepParams &p, const BodyDesc &d, const BodyState *st, f3 body_pos, SCol *cols) {
    f3 lmin = vmin(ld3(st->bmin), ld3(st->pmin)), lmax = vmax(ld3(st->bmax), ld3(st->pmax));
    f3 r3 = mk(d.vertex_radius, d.vertex_radius, d.vertex_radius);
    lmin = lmin - r3;
    lmax = lmax + r3;
    f3 wmin = body_pos + lmin, wmax = body_pos + lmax;
    int n = 0;
    for (uint32_t ci = 0; ci < p.num_colliders; ++ci) {
        const ColliderDev c = p.colliders[ci];
        f3 cp = ld3(c.position);
        // world bounds of the shape (Shape::GetWorldSpaceBounds; CapsuleShape.cpp:266-276 for a capsule)
        f3 cmin, cmax;
        if (c.type == 2) {
            const f3 rr = mk(c.radius, c.radius, c.radius);
            cmin = mk(cp.x, cp.y - c.half_extent[1], cp.z) - rr;
            cmax = mk(cp.x, cp.y + c.half_extent[1], cp.z) + rr;
        } else {
            const f3 ext = c.type == 0 ? ld3(c.half_extent)
                                       : (c.type == 1 ? mk(c.radius, c.radius, c.radius) : mk(c.radius, c.half_extent[1], c.radius));
            cmin = cp + neg(ext);
            cmax = cp + ext;
        }
        bool overlap = !(wmin.x > cmax.x || wmin.y > cmax.y || wmin.z > cmax.z || wmax.x < cmin.x || wmax.y < cmin.y ||
                         wmax.z < cmin.z);
        if (!overlap) continue;
        if (n == int(kMaxCollidingShapes)) {
            atomicOr(p.error, kErrShapeOverflow);
            break;
        }
        SCol &s = cols[n++];
        s.type = c.type;
        s.flags = 0;
        s.isc = 1.0f;
        st3(s.t, cp - body_pos);
        st3(s.h, ld3(c.half_extent));
        s.r = c.radius;
        s.friction = sqrtf(d.friction * c.friction);
        s.restitution = d.restitution > c.restitution ? d.restitution : c.restitution;
    }
    return n;
}

// Host-determined colliding shapes of a body (jsb_body_set_colliding_shapes) into `cols`, with the inverse
// of each transform as Mat44::InversedRotationTranslation computes it (Mat44.inl): the transposed
// rotation and -(R^T t) = 0 - ((c0' t.x + c1' t.y) + c2' t.z). Resets the table's output velocities to the
// input ones. Returns the count; `dynamic` tells whether a dynamic shape is among them.
__device__ inline int load_shape_table(ShapeTable *tb, SCol *cols, bool &dynamic) {
    const int n = int(tb->count < kMaxCollidingShapes ? tb->count : kMaxCollidingShapes);
    dynamic = false;
    for (int k = 0; k < n; ++k) {
        const ShapeEntry &e = tb->e[k];
        SCol &s = cols[k];
        s.type = e.type;
        s.flags = kColRotated | (e.motion == kMotionDynamic ? kColDynamic : 0) | (e.motion == kMotionSensor ? kColSensor : 0);
        dynamic = dynamic || e.motion == kMotionDynamic;
        for (int j = 0; j < 9; ++j) s.c[j] = e.xf[j];
        for (int col = 0; col < 3; ++col)
            for (int row = 0; row < 3; ++row) s.ic[3 * col + row] = e.xf[3 * row + col];
        const f3 t = mk(e.xf[9], e.xf[10], e.xf[11]);
        st3(s.t, t);
        st3(s.it, neg(mat_mul3(s.ic, t)));
        st3(s.h, ld3(e.half_extent));
        s.r = e.radius;
        s.friction = e.friction;
        s.restitution = e.restitution;
        s.isc = e.inv_mass_scale;
        s.hull = int32_t(e.hull);
        for (int j = 0; j < 3; ++j) {
            tb->lin[k][j] = e.lin[j];
            tb->ang[k][j] = e.ang[j];
        }
    }
    tb->updated = 0;
    return n;
}

// UpdateSoftBodyState (:827-921), per-body part: average linear / angular velocity from the vertex sums,
// recentring by the centre of the local bounds when the body position is updated, and the new world
// position (identity rotation; PhysicsSystem.cpp:2864). Returns the recentring offset.
__device__ inline f3 finish_body_state(BodyState *st, const BodyDesc &d, f3 body_pos, f3 bmin, f3 bmax, f3 pmin, f3 pmax,
                                       const float sums[6], float nvf) {
    st3(st->lin_vel, mk(sums[0], sums[1], sums[2]) / nvf);
    st3(st->ang_vel, mk(sums[3], sums[4], sums[5]) / nvf);
    f3 delta = mk(0, 0, 0);
    f3 pos = body_pos;
    if (d.flags & kFlagUpdatePosition) {
        delta = 0.5f * (bmin + bmax);
        f3 nd = neg(delta);
        bmin = bmin + nd;
        bmax = bmax + nd;
        pmin = pmin + nd;
        pmax = pmax + nd;
        f3 wd;
        wd.x = (1.0f * delta.x + 0.0f * delta.y) + 0.0f * delta.z;
        wd.y = (0.0f * delta.x + 1.0f * delta.y) + 0.0f * delta.z;
        wd.z = (0.0f * delta.x + 0.0f * delta.y) + 1.0f * delta.z;
        pos = pos + wd;
    }
    st3(st->bmin, bmin);
    st3(st->bmax, bmax);
    st3(st->pmin, pmin);
    st3(st->pmax, pmax);
    st3(st->position, pos);
    return delta;
}

// Sleeping (SoftBodyMotionProperties.cpp:902-915 with the deactivation of PhysicsSystem.cpp:2875-2884 and
// BodyManager.cpp:559-561), thread 0 after UpdateSoftBodyState: with sleeping allowed, a body whose
// largest squared vertex velocity of the step (before the clamp; NaN values do not count, as with the
// reference's std::max) exceeds the point-velocity threshold restarts its sleep timer; otherwise the
// step's dt is added and, once the timer reaches the time before sleep, the body leaves the active set
// (its body velocities are zeroed) and is not stepped again until woken.
__device__ inline void sleep_test(const StepParams &p, uint32_t b, const BodyDesc &d, BodyState *st, float max_v_sq) {
    if (!p.sleep || !(d.flags & kFlagAllowSleeping)) return;
    BodySleep &s = p.sleep[b];
    if (max_v_sq > p.sleep_velocity_threshold) {
        s.timer = 0.0f;
        return;
    }
    s.timer = s.timer + p.dt;
    if (s.timer >= p.time_before_sleep) {
        s.active = 0u;
        st3(st->lin_vel, mk(0.0f, 0.0f, 0.0f));
        st3(st->ang_vel, mk(0.0f, 0.0f, 0.0f));
    }
}

// Whether body b is stepped (every thread, before anything of the step is written). A body with a force
// this step is woken first, as BodyInterface::AddForce does (EActivation::Activate resets the sleep timer
// and activates the body, BodyInterface.cpp:699-713, BodyManager.cpp:508-522); `wake` is then true and
// thread 0 writes the record after the caller's next barrier.
__device__ __forceinline__ bool body_awake(const StepParams &p, uint32_t b, bool &wake) {
    wake = false;
    if (!p.sleep) return true;
    const f3 f = ld3(p.forces + 3 * size_t(b)), g = ld3(p.step_forces + 3 * size_t(b));
    wake = f.x != 0.0f || f.y != 0.0f || f.z != 0.0f || g.x != 0.0f || g.y != 0.0f || g.z != 0.0f;
    return wake || p.sleep[b].active != 0u;
}

// Block-wide reductions (results in thread 0); S provides float red[32][4] and int redi[32][4].
template <int T, class S>
__device__ __forceinline__ void reduce_minmax4(S &sh, float v[4], int idx[4], const bool is_max[4]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            float ov = __shfl_down_sync(0xffffffffu, v[k], off);
            int oi = __shfl_down_sync(0xffffffffu, idx[k], off);
            if (is_max[k])
                pick_max(v[k], idx[k], ov, oi);
            else
                pick_min(v[k], idx[k], ov, oi);
        }
    }
    if (T > 32) {
        if (lane == 0)
            for (int k = 0; k < 4; ++k) {
                sh.red[warp][k] = v[k];
                sh.redi[warp][k] = idx[k];
            }
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 1; w < T / 32; ++w)
                for (int k = 0; k < 4; ++k) {
                    if (is_max[k])
                        pick_max(v[k], idx[k], sh.red[w][k], sh.redi[w][k]);
                    else
                        pick_min(v[k], idx[k], sh.red[w][k], sh.redi[w][k]);
                }
        __syncthreads();
    }
}

template <int T, class S>
__device__ __forceinline__ float reduce_max(S &sh, float v, int slot) {  // fmaxf: NaN operands are ignored
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, off));
    if (T > 32) {
        if (lane == 0) sh.red[warp][slot] = v;
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 1; w < T / 32; ++w) v = fmaxf(v, sh.red[w][slot]);
        __syncthreads();
    }
    return v;  // valid in thread 0
}

template <int T, class S>
__device__ __forceinline__ float reduce_sum(S &sh, float v, int slot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (T > 32) {
        if (lane == 0) sh.red[warp][slot] = v;
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 1; w < T / 32; ++w) v += sh.red[w][slot];
        __syncthreads();
    }
    return v;  // valid in thread 0
}


// ---------------------------------------------------------------------------------------------
// Bounds of UpdateSoftBodyState (SoftBodyMotionProperties.cpp:852-875)
// ---------------------------------------------------------------------------------------------
// The reference encapsulates vertices in order with AABox::Encapsulate, i.e. Vec3::sMin / sMax, which are
// _mm_min_ps / _mm_max_ps on its deterministic x86 build: per component, m = (m < p) ? m : p. Among
// finite values that is the minimum, later vertices winning ties; a NaN component resets the running
// value (to NaN, then to the next vertex's value). So per component the result is the extreme over the
// vertices after the last one whose component is NaN, or NaN if that is the last vertex. The pass below
// collects (value, index) extremes of vertices with index > skip[c] (skip = -1: all) and the last NaN
// index per component; a body holding NaNs repeats the pass with skip = those indices.
struct Bounds {
    float mm[4], xx[4], pm[4], px[4];  // min / max of positions, min / max of predicted positions
    int mi[4], xi[4], pmi[4], pxi[4];
    int last_nan[6];  // positions x, y, z, predicted x, y, z
};
__device__ __forceinline__ void bounds_init(Bounds &b) {
    for (int k = 0; k < 4; ++k) {
        b.mm[k] = FLT_MAX, b.xx[k] = -FLT_MAX, b.pm[k] = FLT_MAX, b.px[k] = -FLT_MAX;
        b.mi[k] = b.xi[k] = b.pmi[k] = b.pxi[k] = -1;
    }
    for (int k = 0; k < 6; ++k) b.last_nan[k] = -1;
}
__device__ __forceinline__ void bounds_add(Bounds &b, f3 x, f3 pred, int i, const int skip[6]) {
    const float c[6] = {x.x, x.y, x.z, pred.x, pred.y, pred.z};
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (i > skip[k]) {
            pick_min(b.mm[k], b.mi[k], c[k], i);
            pick_max(b.xx[k], b.xi[k], c[k], i);
        }
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (i > skip[3 + k]) {
            pick_min(b.pm[k], b.pmi[k], c[3 + k], i);
            pick_max(b.px[k], b.pxi[k], c[3 + k], i);
        }
#pragma unroll
    for (int k = 0; k < 6; ++k)
        if (c[k] != c[k]) b.last_nan[k] = i;  // vertices arrive in increasing index order per thread
}
template <int T, class S>
__device__ __forceinline__ void bounds_reduce(S &sh, Bounds &b) {
    const bool mins[4] = {false, false, false, false};
    const bool maxs[4] = {true, true, true, true};
    reduce_minmax4<T>(sh, b.mm, b.mi, mins);
    reduce_minmax4<T>(sh, b.xx, b.xi, maxs);
    reduce_minmax4<T>(sh, b.pm, b.pmi, mins);
    reduce_minmax4<T>(sh, b.px, b.pxi, maxs);
}
// Block-wide maximum of the six last-NaN indices, written to out[6] (shared) and visible to every thread.
template <int T>
__device__ __forceinline__ void reduce_last_nan(const int v[6], int *out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int r[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        r[k] = v[k];
        for (int off = 16; off > 0; off >>= 1) r[k] = max(r[k], __shfl_down_sync(0xffffffffu, r[k], off));
    }
    __syncthreads();  // earlier readers of out are done
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; ++k) out[k] = r[k];
    __syncthreads();
    if (T > 32 && lane == 0 && warp > 0)
        for (int k = 0; k < 6; ++k) atomicMax(out + k, r[k]);
    __syncthreads();
}
// Components whose last vertex is NaN end as NaN (the canonical NaN).
__device__ __forceinline__ void bounds_nan_tail(Bounds &b, const int *last_nan, int num_vertices) {
    const float q = __int_as_float(0x7fffffff);
    for (int k = 0; k < 3; ++k) {
        if (last_nan[k] == num_vertices - 1) b.mm[k] = b.xx[k] = q;
        if (last_nan[3 + k] == num_vertices - 1) b.pm[k] = b.px[k] = q;
    }
}

}  // namespace
}  // namespace jsb
