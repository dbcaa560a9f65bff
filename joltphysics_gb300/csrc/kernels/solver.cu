// Soft-body solver step on sm_103a: one CTA advances one body through one full step
// (Jolt/Physics/SoftBody/SoftBodyMotionProperties.cpp: InitializeUpdateContext :937-960,
// DetermineCollidingShapes :120-255, DetermineCollisionPlanes :257-265, N x {ApplyPressure :291-323,
// IntegratePositions :325-365, ParallelApplyConstraints :1057-1115, ApplyCollisionConstraintsAndUpdate-
// Velocities :700-825}, UpdateSoftBodyState :827-921) and PhysicsSystem.cpp:2864 (body position).
//
// The body's positions (+ inverse mass) live in shared memory for the whole step. Constraint
// projection walks a dependency-level schedule built on the host from the update groups and their
// in-group order: constraints in one level touch disjoint vertices (LRA anchors are read-only), so
// projecting a level's constraints concurrently and barrier-separating levels gives the bitwise result
// of the reference's sequential Gauss-Seidel walk. No atomics are involved in the projection.
//
// Bitwise parity with the reference (built with JPH_CROSS_PLATFORM_DETERMINISTIC) needs the
// reference's float operation order: this file is compiled with --fmad=false and IEEE division and
// square root, and the helpers below evaluate Vec3 dot products as (x*x' + y*y') + (z*z' + 0)
// (Jolt/Math/Vec3.inl:896-934), cross products with separately rounded products (:855-895) and
// negation as 0 - x (:669-700).
//
// Persistent launch: the grid holds as many CTAs as fit; each CTA pulls body indices from a work
// queue (an atomic counter over a list sorted by estimated cost, largest first) until it is empty.

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "common.cuh"
#include "device_types.h"

namespace jsb {
namespace {

struct SCol {  // one colliding shape, relative to the soft body
    int32_t type;
    float t[3];
    float h[3];
    float r;
    float friction;
    float restitution;
};

struct Shared {
    SCol cols[kMaxCollidingShapes];
    int ncols;
    uint32_t item;
    float six_volume;
    float delta[3];
    uint4 ring_desc[4];
    float red[32][4];  // per-warp partials for reductions
    int redi[32][4];
};

// ---------------------------------------------------------------------------------------------
// Constraint projections (exact reference arithmetic)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void project_bend(float4 *sx, uint4 r, float inv_dt_sq) {  // :367-456
    uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16, i2 = r.y & 0xffff, i3 = r.y >> 16;
    float compliance = __uint_as_float(r.z), initial_angle = __uint_as_float(r.w);
    float4 p0 = sx[i0], p1 = sx[i1], p2 = sx[i2], p3 = sx[i3];
    f3 x0 = xyz(p0), x1 = xyz(p1), x2 = xyz(p2), x3 = xyz(p3);
    f3 e = x1 - x0;
    float e_len = len(e);
    if (e_len < 1.0e-6f) return;
    f3 x1x2 = x2 - x1, x1x3 = x3 - x1;
    f3 n1 = cross(x2 - x0, x1x2);
    f3 n2 = cross(x1x3, x3 - x0);
    float n1_len_sq = len_sq(n1), n2_len_sq = len_sq(n2);
    float n1n2 = n1_len_sq * n2_len_sq;
    if (n1n2 < 1.0e-24f) return;
    float sign = dot(cross(n2, n1), e) < 0.0f ? -1.0f : 1.0f;
    float d = jdiv(dot(n1, n2), jsqrt(n1n2));
    float c = sign * acos_approximate(d) - initial_angle;
    if (c > kPi)
        c -= 2.0f * kPi;
    else if (c < -kPi)
        c += 2.0f * kPi;
    n1 = n1 / n1_len_sq;
    n2 = n2 / n2_len_sq;
    f3 d0c = (dot(x1x2, e) * n1 + dot(x1x3, e) * n2) / e_len;
    f3 d2c = e_len * n1;
    f3 d3c = e_len * n2;
    f3 d1c = (neg(d0c) - d2c) - d3c;
    float w0 = p0.w, w1 = p1.w, w2 = p2.w, w3 = p3.w;
    float denom = w0 * len_sq(d0c) + w1 * len_sq(d1c) + w2 * len_sq(d2c) + w3 * len_sq(d3c) + compliance * inv_dt_sq;
    if (denom < 1.0e-12f) return;
    float ml = jdiv(c, denom);
    sx[i0] = with_w(x0 - (ml * w0) * d0c, w0);
    sx[i1] = with_w(x1 - (ml * w1) * d1c, w1);
    sx[i2] = with_w(x2 - (ml * w2) * d2c, w2);
    sx[i3] = with_w(x3 - (ml * w3) * d3c, w3);
}

__device__ __forceinline__ void project_volume(float4 *sx, uint4 r, float inv_dt_sq) {  // :458-507
    uint32_t i1 = r.x & 0xffff, i2 = r.x >> 16, i3 = r.y & 0xffff, i4 = r.y >> 16;
    float six_rest = __uint_as_float(r.z), compliance = __uint_as_float(r.w);
    float4 p1 = sx[i1], p2 = sx[i2], p3 = sx[i3], p4 = sx[i4];
    f3 x1 = xyz(p1), x2 = xyz(p2), x3 = xyz(p3), x4 = xyz(p4);
    f3 x1x2 = x2 - x1, x1x3 = x3 - x1, x1x4 = x4 - x1;
    float c = fabsf(dot(cross(x1x2, x1x3), x1x4)) - six_rest;
    f3 d1c = cross(x4 - x2, x3 - x2);
    f3 d2c = cross(x1x3, x1x4);
    f3 d3c = cross(x1x4, x1x2);
    f3 d4c = cross(x1x2, x1x3);
    float w1 = p1.w, w2 = p2.w, w3 = p3.w, w4 = p4.w;
    float denom = w1 * len_sq(d1c) + w2 * len_sq(d2c) + w3 * len_sq(d3c) + w4 * len_sq(d4c) + compliance * inv_dt_sq;
    if (denom < 1.0e-12f) return;
    float ml = jdiv(c, denom);
    sx[i1] = with_w(x1 - (ml * w1) * d1c, w1);
    sx[i2] = with_w(x2 - (ml * w2) * d2c, w2);
    sx[i3] = with_w(x3 - (ml * w3) * d3c, w3);
    sx[i4] = with_w(x4 - (ml * w4) * d4c, w4);
}

__device__ __forceinline__ void project_edge(float4 *sx, uint4 r, float inv_dt_sq) {  // :573-601
    uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16;
    float rest = __uint_as_float(r.z), compliance = __uint_as_float(r.w);
    float4 p0 = sx[i0], p1 = sx[i1];
    f3 x0 = xyz(p0), x1 = xyz(p1);
    f3 delta = x1 - x0;
    float length = len(delta);
    float denom = length * (p0.w + p1.w + compliance * inv_dt_sq);
    if (denom < 1.0e-12f) return;
    f3 corr = (delta * (length - rest)) / denom;
    sx[i0] = with_w(x0 + p0.w * corr, p0.w);
    sx[i1] = with_w(x1 - p1.w * corr, p1.w);
}

__device__ __forceinline__ void project_lra(float4 *sx, uint4 r) {  // :679-698
    uint32_t i0 = r.x & 0xffff, i1 = r.x >> 16;
    float md = __uint_as_float(r.z);
    f3 x0 = xyz(sx[i0]);
    float4 p1 = sx[i1];
    f3 delta = xyz(p1) - x0;
    float dls = len_sq(delta);
    if (dls > md * md) sx[i1] = with_w(x0 + (delta * md) / jsqrt(dls), p1.w);
}

__device__ __forceinline__ void project(float4 *sx, uint4 r, int type, float inv_dt_sq) {
    if (type == 0)
        project_bend(sx, r, inv_dt_sq);
    else if (type == 1)
        project_volume(sx, r, inv_dt_sq);
    else if (type == 2)
        project_edge(sx, r, inv_dt_sq);
    else
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

// Record ring: kRingDepth levels of up to `slots` records each are streamed into shared memory
// ahead of the level being projected; the ring holds kRingDepth + 1 levels.
constexpr int kRingDepth = 3;
constexpr int kRingLevels = kRingDepth + 1;

struct LevelRing {
    uint4 *rec;      // [kRingLevels][slots]
    uint4 *desc;     // [kRingLevels] level descriptors
    uint32_t slots;  // capacity per level
};

// Stages level `idx` (descriptor, and its records when they fit a ring slot) into ring position
// idx % kRingLevels. idx == num_levels stages the sentinel descriptor only.
template <int T>
__device__ __forceinline__ void ring_stage(const LevelRing &ring, const uint4 *__restrict__ levels, const uint4 *__restrict__ rec,
                                           uint32_t idx, uint32_t L, uint4 lv, uint32_t next_first) {
    const uint32_t pos = idx % kRingLevels;
    if (idx < L) {
        const uint32_t n = next_first - lv.x;
        if (n <= ring.slots)
            for (uint32_t s = threadIdx.x; s < n; s += T) cp_async16(ring.rec + pos * ring.slots + s, rec + lv.x + s);
    }
    if (threadIdx.x == 0) ring.desc[pos] = lv;
}

// Walks the dependency levels of one substep. Level l + kRingDepth is staged (cp.async) while level
// l is projected, so the critical path of a level is: descriptor and records from shared memory,
// positions from shared memory, projection, positions to shared memory, barrier.
// Records a constraint's inputs for the adjoint: vertex differences relative to its first vertex
// (edge / LRA: x1 - x0; volume / bend: x2 - x1, x3 - x1, x4 - x1 in record order).
__device__ __forceinline__ void tape_inputs(const float4 *sx, uint4 r, int type, float4 *out) {
    const uint32_t a = r.x & 0xffff, b = r.x >> 16;
    const f3 xa = xyz(sx[a]);
    out[0] = with_w(xyz(sx[b]) - xa, 0.0f);
    if (type <= 1) {
        out[1] = with_w(xyz(sx[r.y & 0xffff]) - xa, 0.0f);
        out[2] = with_w(xyz(sx[r.y >> 16]) - xa, 0.0f);
    }
}

template <int T, bool kTape>
__device__ __forceinline__ void apply_levels(float4 *sx, const BodyDesc &d, float inv_dt_sq, const LevelRing &ring,
                                             float4 *tape_cons) {
    const uint4 *__restrict__ levels = d.levels;
    const uint4 *__restrict__ rec = d.records;
    const uint32_t tid = threadIdx.x;
    const uint32_t L = d.num_levels;
    if (L == 0) return;
    // prologue: stage levels 0 .. kRingDepth - 1 (levels has L + 2 entries)
#pragma unroll
    for (int k = 0; k < kRingDepth; ++k) {
        if (uint32_t(k) <= L) ring_stage<T>(ring, levels, rec, k, L, __ldg(levels + k), __ldg(levels + k + 1).x);
        cp_async_commit();
    }
    cp_async_wait<kRingDepth - 1>();
    __syncthreads();
    for (uint32_t l = 0; l < L; ++l) {
        const uint32_t ahead = l + kRingDepth;
        uint4 lv_ahead = make_uint4(0, 0, 0, 0);
        uint32_t next_ahead = 0;
        if (ahead <= L) {
            lv_ahead = __ldg(levels + ahead);
            next_ahead = __ldg(levels + ahead + 1).x;
        }
        const uint32_t pos = l % kRingLevels;
        const uint4 lv = ring.desc[pos];
        const uint32_t n = ring.desc[(l + 1) % kRingLevels].x - lv.x;
        const bool in_ring = n <= ring.slots;
        const uint4 *src = in_ring ? ring.rec + pos * ring.slots : rec + lv.x;
        for (uint32_t s = tid; s < n; s += T) {
            const uint4 r = src[s];
            if (r.x != 0xffffffffu) {
                if (kTape) tape_inputs(sx, r, slot_type(lv, s), tape_cons + size_t(lv.x + s) * 3);
                project(sx, r, slot_type(lv, s), inv_dt_sq);
            }
        }
        if (ahead <= L) ring_stage<T>(ring, levels, rec, ahead, L, lv_ahead, next_ahead);
        cp_async_commit();
        cp_async_wait<kRingDepth - 1>();
        cta_sync<T>();
    }
    cp_async_wait<0>();
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

// BoxShape::CollideSoftBodyVertices (BoxShape.cpp:234-283) for one vertex.
__device__ __forceinline__ void collide_box(f3 p, const SCol &s, int idx, float &largest, float4 &plane, int &shape) {
    f3 t = ld3(s.t), h = ld3(s.h);
    f3 local = p + neg(t);
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
        plane = plane_transformed(normal, point, t);
        shape = idx;
    } else {
        f3 normal = local - clamped;
        float nl = len(normal);
        float pen = -nl;
        if (largest >= pen) return;
        largest = pen;
        normal = normal / nl;
        plane = plane_transformed(normal, clamped, t);
        shape = idx;
    }
}

// SphereShape::CollideSoftBodyVertices (SphereShape.cpp:279-300) for one vertex.
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

template <int T>
__device__ __forceinline__ void reduce_minmax4(Shared &sh, float v[4], int idx[4], const bool is_max[4]) {
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

template <int T>
__device__ __forceinline__ float reduce_sum(Shared &sh, float v, int slot) {
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
// One body, one step
// ---------------------------------------------------------------------------------------------
// Shared memory of one CTA (dynamic part), cap = the launch's largest vertex count:
//   kSmemState:  x[cap] | v[cap] (shape index in v.w) | prev[cap] | faces[...]
//   otherwise:   x[cap] | faces[...]       (v, prev, shape stay in HBM)
// faces: per-face triple product, then per-face pressure impulse (pressure bodies only).
template <int T, bool kSmemState, bool kTape = false>
__device__ void step_body(const StepParams &p, uint32_t b, float4 *smem, uint32_t cap, Shared &sh) {
    const uint32_t tid = threadIdx.x;
    const BodyDesc d = p.bodies[b];
    BodyState *st = p.states + b;
    const uint32_t nv = d.num_vertices;
    float4 *__restrict__ gx = p.x + d.vtx_offset;
    float4 *__restrict__ gv = p.v + d.vtx_offset;
    float4 *__restrict__ gprev = p.prev + d.vtx_offset;
    float4 *__restrict__ gplane = p.plane + d.vtx_offset;
    int32_t *__restrict__ gshape = p.shape + d.vtx_offset;
    float4 *sx = smem;
    float4 *sv = smem + cap;
    float4 *sprev = smem + 2 * cap;
    float4 *sface = smem + (kSmemState ? 3 * cap : cap);  // pressure faces; the record ring reuses it
    TapeDesc td = {};
    if (kTape) td = p.tape[b];
    LevelRing ring;
    ring.rec = reinterpret_cast<uint4 *>(sface);
    ring.desc = sh.ring_desc;
    ring.slots = p.ring_slots;

    // InitializeUpdateContext (identity body rotation)
    const f3 g = d.gravity_factor * ld3(p.gravity);
    const uint32_t n_it = d.num_iterations;
    const float dt = p.dt;
    const float dt_sub = dt / float(n_it);
    float disp_scale = 0.5f * float(n_it);
    disp_scale = disp_scale * float(n_it + 1);
    disp_scale = disp_scale * (dt_sub * dt_sub);
    const f3 disp_g = disp_scale * g;
    const f3 body_pos = ld3(st->position);
    const f3 force = ld3(p.forces + 3 * size_t(b)) + ld3(p.step_forces + 3 * size_t(b));

    // DetermineCollidingShapes: world AABB of (bounds U predicted bounds) grown by the vertex radius
    if (tid == 0) {
        f3 lmin = vmin(ld3(st->bmin), ld3(st->pmin)), lmax = vmax(ld3(st->bmax), ld3(st->pmax));
        f3 r3 = mk(d.vertex_radius, d.vertex_radius, d.vertex_radius);
        lmin = lmin - r3;
        lmax = lmax + r3;
        f3 wmin = body_pos + lmin, wmax = body_pos + lmax;
        int n = 0;
        for (uint32_t ci = 0; ci < p.num_colliders; ++ci) {
            const ColliderDev c = p.colliders[ci];
            f3 cp = ld3(c.position);
            f3 ext = c.type == 0 ? ld3(c.half_extent) : mk(c.radius, c.radius, c.radius);
            f3 cmin = cp + neg(ext), cmax = cp + ext;
            bool overlap = !(wmin.x > cmax.x || wmin.y > cmax.y || wmin.z > cmax.z || wmax.x < cmin.x || wmax.y < cmin.y ||
                             wmax.z < cmin.z);
            if (!overlap) continue;
            if (n == int(kMaxCollidingShapes)) {
                atomicOr(p.error, kErrShapeOverflow);
                break;
            }
            SCol &s = sh.cols[n++];
            s.type = c.type;
            st3(s.t, cp - body_pos);
            st3(s.h, ld3(c.half_extent));
            s.r = c.radius;
            s.friction = sqrtf(d.friction * c.friction);
            s.restitution = d.restitution > c.restitution ? d.restitution : c.restitution;
        }
        sh.ncols = n;
        if (kTape)
            for (int k = 0; k < n; ++k)
                td.cols[size_t(p.tape_step) * kMaxCollidingShapes + k] = make_float2(sh.cols[k].friction, sh.cols[k].restitution);
    }
    // Stage the state in shared memory.
    for (uint32_t i = tid; i < nv; i += T) {
        sx[i] = gx[i];
        if (kSmemState) sv[i] = gv[i];
    }
    __syncthreads();

    // DetermineCollisionPlanes (per vertex, once per step)
    const int ncols = sh.ncols;
    for (uint32_t i = tid; i < nv; i += T) {
        float4 pi = sx[i];
        int shape = -1;
        float4 plane = make_float4(0, 0, 0, 0);
        if (pi.w > 0.0f && ncols > 0) {
            float largest = -FLT_MAX;
            for (int s = 0; s < ncols; ++s) {
                if (sh.cols[s].type == 0)
                    collide_box(xyz(pi), sh.cols[s], s, largest, plane, shape);
                else
                    collide_sphere(xyz(pi), sh.cols[s], s, largest, plane, shape);
            }
        }
        if (kSmemState)
            sv[i].w = __int_as_float(shape);
        else
            gshape[i] = shape;
        if (shape >= 0) gplane[i] = plane;
        if (kTape) {
            td.plane[size_t(p.tape_step) * nv + i] = plane;
            td.shape[size_t(p.tape_step) * nv + i] = shape;
        }
    }

    const float inv_dt_sq = 1.0f / (dt_sub * dt_sub);
    float damp = 1.0f - d.linear_damping * dt_sub;
    damp = damp < 0.0f ? 0.0f : damp;
    const f3 sub_g = g * dt_sub;
    const float nvf = float(nv > 0 ? nv : 1);
    const f3 sub_imp = (force * dt_sub) / nvf;
    const float restitution_threshold = -2.0f * len(g) * dt_sub;
    const bool has_pressure = d.pressure > 0.0f && d.num_faces > 0;

    for (uint32_t it = 0; it < n_it; ++it) {
        float4 *tape_state = nullptr;
        if (kTape) {
            tape_state = td.state + (size_t(p.tape_step) * n_it + it) * 3 * nv;
            for (uint32_t i = tid; i < nv; i += T) tape_state[i] = sx[i];
        }
        // ApplyPressure
        if (has_pressure) {
            float *s_six = reinterpret_cast<float *>(sface);
            for (uint32_t f = tid; f < d.num_faces; f += T) {
                uint4 fc = __ldg(d.faces + f);
                s_six[f] = dot(cross(xyz(sx[fc.x]), xyz(sx[fc.y])), xyz(sx[fc.z]));
            }
            __syncthreads();
            if (tid == 0) {  // the reference sums the faces sequentially
                float six = 0.0f;
                for (uint32_t f = 0; f < d.num_faces; ++f) six = six + s_six[f];
                sh.six_volume = six;
            }
            __syncthreads();
            const float six = sh.six_volume;
            if (six > 0.0f) {
                const float coefficient = jdiv(d.pressure * dt_sub, six);
                for (uint32_t f = tid; f < d.num_faces; f += T) {
                    uint4 fc = __ldg(d.faces + f);
                    f3 x1 = xyz(sx[fc.x]), x2 = xyz(sx[fc.y]), x3 = xyz(sx[fc.z]);
                    sface[f] = with_w(coefficient * cross(x2 - x1, x3 - x1), 0.0f);
                }
                __syncthreads();
                for (uint32_t i = tid; i < nv; i += T) {
                    const float w = sx[i].w;
                    float4 vel = kSmemState ? sv[i] : gv[i];
                    f3 v = xyz(vel);
                    for (uint32_t k = __ldg(d.vf_off + i), ke = __ldg(d.vf_off + i + 1); k < ke; ++k)
                        v = v + w * xyz(sface[__ldg(d.vf + k)]);
                    if (kSmemState)
                        sv[i] = with_w(v, vel.w);
                    else
                        gv[i] = with_w(v, vel.w);
                }
            }
            __syncthreads();
        }
        // IntegratePositions
        for (uint32_t i = tid; i < nv; i += T) {
            float4 pi = sx[i];
            float4 vel = kSmemState ? sv[i] : gv[i];
            f3 v = xyz(vel);
            if (pi.w > 0.0f) {
                v = v + (sub_g + sub_imp * pi.w);
                v = v * damp;
            }
            if (kSmemState) {
                sprev[i] = pi;
                sv[i] = with_w(v, vel.w);
            } else {
                gprev[i] = pi;
                gv[i] = with_w(v, vel.w);
            }
            sx[i] = with_w(xyz(pi) + v * dt_sub, pi.w);
            if (kTape) tape_state[nv + i] = with_w(v, 0.0f);
        }
        __syncthreads();
        // Update groups in dependency-level order
        apply_levels<T, kTape>(sx, d, inv_dt_sq, ring,
                               kTape ? td.cons + (size_t(p.tape_step) * n_it + it) * size_t(td.slots) * 3 : nullptr);
        __syncthreads();
        if (kTape)
            for (uint32_t i = tid; i < nv; i += T) tape_state[2 * nv + i] = sx[i];
        // ApplyCollisionConstraintsAndUpdateVelocities (static colliders)
        for (uint32_t i = tid; i < nv; i += T) {
            float4 pi = sx[i];
            if (!(pi.w > 0.0f)) continue;
            f3 x = xyz(pi);
            float4 vel = kSmemState ? sv[i] : gv[i];
            float4 prev = kSmemState ? sprev[i] : gprev[i];
            f3 prev_v = xyz(vel);
            f3 v = (x - xyz(prev)) / dt_sub;
            int shape = -1;
            if (ncols > 0) shape = kSmemState ? __float_as_int(vel.w) : gshape[i];
            if (shape >= 0) {
                float4 pl = gplane[i];
                f3 n = xyz(pl);
                float projected = -(dot(x, n) + pl.w) + d.vertex_radius;
                if (projected > 0.0f) {
                    const SCol &cs = sh.cols[shape];
                    x = x + n * projected;
                    sx[i] = with_w(x, pi.w);
                    f3 v_normal = n * dot(n, v);
                    f3 v_tan = v - v_normal;
                    float vtl = len(v_tan);
                    if (vtl > 0.0f) {
                        float fr = jdiv(cs.friction * projected, vtl * dt_sub);
                        fr = fr > 1.0f ? 1.0f : fr;
                        v = v - v_tan * fr;
                    }
                    v = v - v_normal;
                    float pvn = dot(prev_v, n);
                    if (pvn < restitution_threshold) v = v - (cs.restitution * pvn) * n;
                }
            }
            if (kSmemState)
                sv[i] = with_w(v, vel.w);
            else
                gv[i] = with_w(v, vel.w);
        }
        __syncthreads();
    }

    // UpdateSoftBodyState
    const float max_sq = d.max_linear_velocity * d.max_linear_velocity;
    float mm[4] = {FLT_MAX, FLT_MAX, FLT_MAX, 0};
    int mi[4] = {-1, -1, -1, -1};
    float xx[4] = {-FLT_MAX, -FLT_MAX, -FLT_MAX, 0};
    int xi[4] = {-1, -1, -1, -1};
    float pm[4] = {FLT_MAX, FLT_MAX, FLT_MAX, 0};
    int pmi[4] = {-1, -1, -1, -1};
    float px[4] = {-FLT_MAX, -FLT_MAX, -FLT_MAX, 0};
    int pxi[4] = {-1, -1, -1, -1};
    f3 lin = mk(0, 0, 0), ang = mk(0, 0, 0);
    bool finite = true;
    for (uint32_t i = tid; i < nv; i += T) {
        float4 pi = sx[i];
        float4 vel = kSmemState ? sv[i] : gv[i];
        f3 v = xyz(vel), x = xyz(pi);
        float vsq = len_sq(v);
        if (vsq > max_sq) v = v * jsqrt(jdiv(max_sq, vsq));
        gv[i] = with_w(v, 0.0f);
        lin = lin + v;
        ang = ang + cross(x, v);
        f3 pred = (x + v * dt) + disp_g;
        pick_min(mm[0], mi[0], x.x, int(i));
        pick_min(mm[1], mi[1], x.y, int(i));
        pick_min(mm[2], mi[2], x.z, int(i));
        pick_max(xx[0], xi[0], x.x, int(i));
        pick_max(xx[1], xi[1], x.y, int(i));
        pick_max(xx[2], xi[2], x.z, int(i));
        pick_min(pm[0], pmi[0], pred.x, int(i));
        pick_min(pm[1], pmi[1], pred.y, int(i));
        pick_min(pm[2], pmi[2], pred.z, int(i));
        pick_max(px[0], pxi[0], pred.x, int(i));
        pick_max(px[1], pxi[1], pred.y, int(i));
        pick_max(px[2], pxi[2], pred.z, int(i));
        finite = finite && isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
    }
    if (!finite) atomicOr(p.error, kErrNonFinite);
    {
        const bool mins[4] = {false, false, false, false};
        const bool maxs[4] = {true, true, true, true};
        reduce_minmax4<T>(sh, mm, mi, mins);
        reduce_minmax4<T>(sh, xx, xi, maxs);
        reduce_minmax4<T>(sh, pm, pmi, mins);
        reduce_minmax4<T>(sh, px, pxi, maxs);
    }
    float sums[6];
    sums[0] = reduce_sum<T>(sh, lin.x, 0);
    sums[1] = reduce_sum<T>(sh, lin.y, 1);
    sums[2] = reduce_sum<T>(sh, lin.z, 2);
    sums[3] = reduce_sum<T>(sh, ang.x, 3);
    sums[4] = reduce_sum<T>(sh, ang.y, 0);
    sums[5] = reduce_sum<T>(sh, ang.z, 1);
    if (tid == 0) {
        f3 bmin = mk(mm[0], mm[1], mm[2]), bmax = mk(xx[0], xx[1], xx[2]);
        f3 pmin = mk(pm[0], pm[1], pm[2]), pmax = mk(px[0], px[1], px[2]);
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
        st3(sh.delta, delta);
    }
    __syncthreads();
    const f3 delta = ld3(sh.delta);
    const bool shift = (d.flags & kFlagUpdatePosition) != 0;
    for (uint32_t i = tid; i < nv; i += T) {
        float4 pi = sx[i];
        gx[i] = shift ? with_w(xyz(pi) - delta, pi.w) : pi;
    }
    __syncthreads();
}

template <int T, bool kSmemState, bool kTape = false>
__global__ void __launch_bounds__(T) step_kernel(StepParams p, uint32_t cap) {
    extern __shared__ float4 smem[];
    __shared__ Shared sh;
    for (;;) {
        if (threadIdx.x == 0) sh.item = atomicAdd(p.queue, 1u);
        __syncthreads();
        const uint32_t item = sh.item;
        __syncthreads();
        if (item >= p.num_work) return;
        step_body<T, kSmemState, kTape>(p, p.work[item], smem, cap, sh);
    }
}

}  // namespace

// Bytes of dynamic shared memory for a launch whose largest body has `vertices` vertices and whose
// largest pressurised body has `faces` faces.
size_t step_smem_bytes(bool smem_state, uint32_t vertices, uint32_t faces, uint32_t ring_slots) {
    const size_t faces_bytes = size_t(faces) * sizeof(float4);
    const size_t ring_bytes = size_t(kRingLevels) * ring_slots * sizeof(uint4);
    return size_t(vertices) * sizeof(float4) * (smem_state ? 3 : 1) + (faces_bytes > ring_bytes ? faces_bytes : ring_bytes);
}

#define JSB_FOR_EACH_SHAPE(X) X(32, true) X(64, true) X(128, true) X(256, true) X(32, false) X(64, false) X(128, false) X(256, false)

// Launches one persistent step over `p.num_work` bodies with `threads` threads per CTA.
cudaError_t launch_step(const StepParams &p, int threads, bool smem_state, uint32_t smem_vertices, uint32_t smem_faces, int grid,
                        cudaStream_t stream) {
    size_t smem = step_smem_bytes(smem_state, smem_vertices, smem_faces, p.ring_slots);
#define JSB_LAUNCH(TT, SS)                                                      \
    if (threads == TT && smem_state == SS) {                                    \
        step_kernel<TT, SS><<<grid, TT, smem, stream>>>(p, smem_vertices);      \
        return cudaGetLastError();                                              \
    }
    JSB_FOR_EACH_SHAPE(JSB_LAUNCH)
#undef JSB_LAUNCH
    return cudaErrorInvalidValue;
}

// Taped forward step (differentiable runs): 128 threads per CTA, every body of the launch.
cudaError_t launch_step_tape(const StepParams &p, bool smem_state, uint32_t smem_vertices, uint32_t smem_faces, int grid,
                             cudaStream_t stream) {
    size_t smem = step_smem_bytes(smem_state, smem_vertices, smem_faces, p.ring_slots);
    if (smem_state)
        step_kernel<128, true, true><<<grid, 128, smem, stream>>>(p, smem_vertices);
    else
        step_kernel<128, false, true><<<grid, 128, smem, stream>>>(p, smem_vertices);
    return cudaGetLastError();
}

int step_tape_occupancy(bool smem_state, size_t smem) {
    int n = 0;
    if (smem_state)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel<128, true, true>, 128, smem);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel<128, false, true>, 128, smem);
    return n;
}

// Allows every solver kernel instance to use up to `max_dynamic_smem` bytes of dynamic shared memory
// (done once per device, outside any stream capture).
cudaError_t init_step_kernels(int max_dynamic_smem) {
    cudaError_t e = cudaSuccess;
#define JSB_ATTR(TT, SS) \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(step_kernel<TT, SS>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem);
    JSB_FOR_EACH_SHAPE(JSB_ATTR)
#undef JSB_ATTR
    if (e == cudaSuccess) e = cudaFuncSetAttribute(step_kernel<128, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(step_kernel<128, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem);
    return e;
}

// Occupancy of step_kernel (CTAs per SM) for a launch shape and dynamic shared memory size.
int step_occupancy(int threads, bool smem_state, size_t smem) {
    int n = 0;
#define JSB_OCC(TT, SS) \
    if (threads == TT && smem_state == SS) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel<TT, SS>, TT, smem);
    JSB_FOR_EACH_SHAPE(JSB_OCC)
#undef JSB_OCC
    return n;
}

}  // namespace jsb

// =============================================================================================
// Allocation-free single-body step (jsb_step_body_noalloc)
// =============================================================================================
// For callers that cannot call cudaMalloc (engines whose device memory all comes from their own
// fixed arenas, frame loops that must not pay a device allocation's implicit synchronisation): the
// step kernel's scratch -- the body's constraint schedule, previous positions, collision planes and
// shape indices -- lives in the static array below instead of context buffers. The caller owns the
// inputs and outputs (vertex state, body record, error word) in its own device memory.

#include <mutex>
#include <string>
#include <vector>

#include "../../../include/jsb.h"
#include "../host/schedule.h"

namespace jsb {

jsb_status report_error(jsb_status code, const std::string &msg);

namespace noalloc {

constexpr uint32_t kMaxVertices = JSB_NOALLOC_MAX_VERTICES;
constexpr uint32_t kMaxSlots = JSB_NOALLOC_MAX_SLOTS;
constexpr uint32_t kMaxLevels = JSB_NOALLOC_MAX_LEVELS;
constexpr uint32_t kMaxFaces = JSB_NOALLOC_MAX_FACES;
constexpr uint32_t kMaxColliders = JSB_NOALLOC_MAX_COLLIDERS;
static_assert(kMaxColliders <= kMaxCollidingShapes, "collider limit");

// Layout of the scratch array, in float4 units.
constexpr size_t kOffPrev = 0;
constexpr size_t kOffPlane = kOffPrev + kMaxVertices;
constexpr size_t kOffShape = kOffPlane + kMaxVertices;             // int32[kMaxVertices]
constexpr size_t kOffLevels = kOffShape + kMaxVertices / 4;        // uint4[kMaxLevels + 2]
constexpr size_t kOffRecords = kOffLevels + kMaxLevels + 2;        // uint4[kMaxSlots]
constexpr size_t kOffFaces = kOffRecords + kMaxSlots;              // uint4[kMaxFaces]
constexpr size_t kOffVfOff = kOffFaces + kMaxFaces;                // uint32[kMaxVertices + 4]
constexpr size_t kOffVf = kOffVfOff + (kMaxVertices + 4) / 4;      // uint32[3 * kMaxFaces]
constexpr size_t kScratchFloat4 = kOffVf + (3 * kMaxFaces) / 4;    // about 2.3 MB

static __device__ __align__(256) float4 g_scratch[kScratchFloat4];

struct Params {
    BodyDesc desc;
    BodyState *state;
    float4 *x, *v;
    float4 *prev, *plane;
    int32_t *shape;
    ColliderDev colliders[kMaxColliders];
    uint32_t num_colliders;
    float gravity[3];
    float dt;
    float force[3];
    float zero3[3];
    uint32_t zero_work;
    uint32_t *error;
};

template <int T, bool kSmemState>
__global__ void __launch_bounds__(T) step_kernel_noalloc(const __grid_constant__ Params q, uint32_t cap) {
    extern __shared__ float4 smem[];
    __shared__ Shared sh;
    StepParams p;
    p.bodies = &q.desc;
    p.states = q.state;
    p.work = &q.zero_work;
    p.num_work = 1;
    p.queue = nullptr;
    p.x = q.x;
    p.v = q.v;
    p.prev = q.prev;
    p.plane = q.plane;
    p.shape = q.shape;
    p.colliders = q.colliders;
    p.num_colliders = q.num_colliders;
    p.gravity[0] = q.gravity[0];
    p.gravity[1] = q.gravity[1];
    p.gravity[2] = q.gravity[2];
    p.dt = q.dt;
    p.error = q.error;
    p.forces = q.force;
    p.step_forces = q.zero3;
    p.ring_slots = 256;
    step_body<T, kSmemState>(p, 0, smem, cap, sh);
}

constexpr int kThreads = 128;
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
float4 *g_scratch_ptr[kMaxDevices] = {};
size_t g_smem_limit[kMaxDevices] = {};

// Once per device, with that device current: the device address of the scratch array (a host-side
// reference to g_scratch is not a device address) and the kernel's dynamic shared memory limit.
jsb_status setup(int device, float4 **scratch, size_t *smem_limit) {
    if (device < 0 || device >= kMaxDevices) return report_error(JSB_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
        if (e != cudaSuccess || !ptr)
            return report_error(JSB_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        int optin = 0;
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
        if (e != cudaSuccess) return report_error(JSB_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
        const int limit = optin - 4096;
        e = cudaFuncSetAttribute(step_kernel_noalloc<kThreads, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(step_kernel_noalloc<kThreads, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
        if (e != cudaSuccess) return report_error(JSB_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
        g_smem_limit[device] = size_t(limit);
        g_scratch_ptr[device] = static_cast<float4 *>(ptr);
    }
    *scratch = g_scratch_ptr[device];
    *smem_limit = g_smem_limit[device];
    return JSB_OK;
}

}  // namespace noalloc
}  // namespace jsb

extern "C" jsb_status jsb_step_body_noalloc(const void *settings_blob, size_t len, const jsb_creation_settings *creation,
                                            const jsb_collider *colliders, uint32_t num_colliders, const float gravity[3],
                                            const float force[3], float dt, void *x_device, void *v_device,
                                            jsb_body_state *state_device, uint32_t *error_device, jsb_stream stream) {
    using namespace jsb;
    using namespace jsb::noalloc;
    static_assert(sizeof(jsb_body_state) == sizeof(BodyState), "jsb_body_state layout");
    if (!settings_blob || !creation || !gravity || !x_device || !v_device || !state_device || !error_device ||
        (num_colliders && !colliders))
        return report_error(JSB_ERR_INVALID_ARGUMENT, "null argument");
    if (!(dt > 0.0f) || creation->num_iterations < 1)
        return report_error(JSB_ERR_INVALID_ARGUMENT, "dt must be > 0 and num_iterations >= 1");
    if (!creation->make_rotation_identity)
        return report_error(JSB_ERR_UNSUPPORTED, "bodies must keep an identity rotation (mMakeRotationIdentity = true)");
    if (num_colliders > kMaxColliders)
        return report_error(JSB_ERR_CAPACITY, "jsb_step_body_noalloc takes at most " + std::to_string(kMaxColliders) + " colliders");

    // Host side: parse the settings and build the padded dependency-level schedule.
    ParsedSettings ps;
    bool unsupported = false;
    std::string err = parse_settings(settings_blob, len, ps, unsupported);
    if (!err.empty()) return report_error(unsupported ? JSB_ERR_UNSUPPORTED : JSB_ERR_BLOB, err);
    const uint32_t nv = uint32_t(ps.vertices.size());
    const bool pressure = creation->pressure > 0.0f;
    const uint32_t nf = pressure ? uint32_t(ps.faces.size()) : 0u;
    if (nv > kMaxVertices)
        return report_error(JSB_ERR_CAPACITY, "body has " + std::to_string(nv) + " vertices; jsb_step_body_noalloc handles at most " +
                                                  std::to_string(kMaxVertices));
    if (nf > kMaxFaces)
        return report_error(JSB_ERR_CAPACITY, "body has " + std::to_string(nf) + " pressure faces; jsb_step_body_noalloc handles at most " +
                                                  std::to_string(kMaxFaces));
    Schedule sched = build_schedule(ps);
    if (sched.num_slots > kMaxSlots || sched.num_levels > kMaxLevels)
        return report_error(JSB_ERR_CAPACITY, "constraint schedule of " + std::to_string(sched.num_slots) + " slots / " +
                                                  std::to_string(sched.num_levels) + " levels exceeds jsb_step_body_noalloc's " +
                                                  std::to_string(kMaxSlots) + " / " + std::to_string(kMaxLevels));
    std::vector<uint32_t> vf_off(nv + 1, 0), vf;
    std::vector<uint4> faces;
    if (pressure) {
        for (const auto &f : ps.faces)
            for (int k = 0; k < 3; ++k) vf_off[f.v[k] + 1]++;
        for (uint32_t i = 0; i < nv; ++i) vf_off[i + 1] += vf_off[i];
        vf.resize(vf_off[nv]);
        std::vector<uint32_t> fill(vf_off.begin(), vf_off.end() - 1);
        for (uint32_t fi = 0; fi < nf; ++fi)
            for (int k = 0; k < 3; ++k) vf[fill[ps.faces[fi].v[k]]++] = fi;
        faces.resize(nf);
        for (uint32_t fi = 0; fi < nf; ++fi) faces[fi] = make_uint4(ps.faces[fi].v[0], ps.faces[fi].v[1], ps.faces[fi].v[2], 0);
    }

    // Device side: scratch address (set-up on the first call on this device), then stage the schedule.
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return report_error(JSB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    float4 *scratch = nullptr;
    size_t smem_limit = 0;
    jsb_status st = setup(device, &scratch, &smem_limit);
    if (st != JSB_OK) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    auto copy = [&](size_t off_float4, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(scratch + off_float4, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    e = copy(kOffLevels, sched.padded_levels.data(), sched.padded_levels.size() * sizeof(uint32_t));
    if (e == cudaSuccess) e = copy(kOffRecords, sched.padded_records.data(), sched.padded_records.size() * sizeof(uint32_t));
    if (e == cudaSuccess && pressure) e = copy(kOffFaces, faces.data(), faces.size() * sizeof(uint4));
    if (e == cudaSuccess && pressure) e = copy(kOffVfOff, vf_off.data(), vf_off.size() * sizeof(uint32_t));
    if (e == cudaSuccess && pressure) e = copy(kOffVf, vf.data(), vf.size() * sizeof(uint32_t));
    if (e != cudaSuccess) return report_error(JSB_ERR_CUDA, std::string("cudaMemcpyAsync(schedule): ") + cudaGetErrorString(e));

    Params q = {};
    BodyDesc &d = q.desc;
    d.levels = reinterpret_cast<const uint4 *>(scratch + kOffLevels);
    d.records = reinterpret_cast<const uint4 *>(scratch + kOffRecords);
    d.faces = reinterpret_cast<const uint4 *>(scratch + kOffFaces);
    d.vf_off = reinterpret_cast<const uint32_t *>(scratch + kOffVfOff);
    d.vf = reinterpret_cast<const uint32_t *>(scratch + kOffVf);
    d.num_levels = sched.num_levels;
    d.num_records = sched.num_slots;
    d.num_faces = pressure ? nf : 0u;
    d.num_vertices = nv;
    d.vtx_offset = 0;
    d.num_iterations = creation->num_iterations;
    d.linear_damping = creation->linear_damping;
    d.max_linear_velocity = creation->max_linear_velocity;
    d.restitution = creation->restitution;
    d.friction = creation->friction;
    d.pressure = creation->pressure;
    d.gravity_factor = creation->gravity_factor;
    d.vertex_radius = creation->vertex_radius;
    d.flags = creation->update_position ? kFlagUpdatePosition : 0u;
    q.state = reinterpret_cast<BodyState *>(state_device);
    q.x = static_cast<float4 *>(x_device);
    q.v = static_cast<float4 *>(v_device);
    q.prev = scratch + kOffPrev;
    q.plane = scratch + kOffPlane;
    q.shape = reinterpret_cast<int32_t *>(scratch + kOffShape);
    for (uint32_t i = 0; i < num_colliders; ++i) {
        ColliderDev &c = q.colliders[i];
        c.type = colliders[i].type;
        for (int k = 0; k < 3; ++k) {
            c.position[k] = colliders[i].position[k];
            c.half_extent[k] = colliders[i].half_extent[k];
        }
        c.radius = colliders[i].radius;
        c.friction = colliders[i].friction;
        c.restitution = colliders[i].restitution;
    }
    q.num_colliders = num_colliders;
    for (int k = 0; k < 3; ++k) {
        q.gravity[k] = gravity[k];
        q.force[k] = force ? force[k] : 0.0f;
        q.zero3[k] = 0.0f;
    }
    q.dt = dt;
    q.zero_work = 0;
    q.error = error_device;

    // Whole vertex state in shared memory when it fits, else positions only (as in the batched path).
    const uint32_t ring_slots = 256;
    const bool smem_state = step_smem_bytes(true, nv, nf, ring_slots) <= smem_limit;
    const size_t smem = step_smem_bytes(smem_state, nv, nf, ring_slots);
    if (smem > smem_limit)
        return report_error(JSB_ERR_UNSUPPORTED, "body does not fit the shared-memory solver path");
    if (smem_state)
        step_kernel_noalloc<kThreads, true><<<1, kThreads, smem, s>>>(q, nv);
    else
        step_kernel_noalloc<kThreads, false><<<1, kThreads, smem, s>>>(q, nv);
    e = cudaGetLastError();
    if (e != cudaSuccess) return report_error(JSB_ERR_CUDA, std::string("step_kernel_noalloc: ") + cudaGetErrorString(e));
    return JSB_OK;
}
