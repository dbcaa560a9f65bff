// Soft-body step for bodies too large for one CTA's shared memory (up to 65,536 vertices): one
// thread-block cluster advances one body through one full step (the same reference functions as
// solver.cu: SoftBodyMotionProperties.cpp InitializeUpdateContext :937-960, DetermineCollidingShapes
// :120-255, DetermineCollisionPlanes :257-265, N x {IntegratePositions :325-365,
// ParallelApplyConstraints :1057-1115, ApplyCollisionConstraintsAndUpdateVelocities :700-825},
// UpdateSoftBodyState :827-921).
//
// Vertex ownership: CTA r of the cluster owns vertices [r << shift, (r + 1) << shift) and keeps their
// positions (+ inverse mass) in its shared memory for the whole step; velocities, previous positions,
// planes and shape indices of its vertices stay in HBM (they are touched once per substep, by the
// owner, coalesced). A constraint reads and writes its vertices wherever they live through distributed
// shared memory (mapa + ld/st.shared::cluster). Every dependency level ends at a cluster barrier
// (arrive.release / wait.acquire), so the level schedule gives the same bitwise result as the one-CTA
// solver and as the reference's sequential Gauss-Seidel walk.
//
// Level slots are dealt round-robin over all threads of the cluster. Each thread streams the records
// it will project a few levels ahead into its own slice of a shared-memory ring with cp.async, so no
// barrier is needed for the ring: a thread only waits for its own copies. The level descriptors are
// copied into shared memory once per step.
//
// Pressure (ApplyPressure): the per-face terms are dealt over the cluster and summed in face order by
// one thread, through a per-body face scratch in HBM. The taped (differentiable) step does not run here.

#include <cuda_runtime.h>
#include <float.h>
#include <stddef.h>
#include <stdint.h>

#include "common.cuh"
#include "device_types.h"
#include "projection.cuh"

namespace jsb {
namespace {

// ---- cluster primitives ------------------------------------------------------------------------
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_size() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }
// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t map_rank(uint32_t local, uint32_t rank) {
    uint32_t out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(local), "r"(rank));
    return out;
}
__device__ __forceinline__ float ld_cluster_f32(uint32_t addr) {
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ int ld_cluster_s32(uint32_t addr) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
    return v;
}

// Position store spread over the cluster: vertex i is at offset (i & mask) of CTA (i >> shift).
struct ClusterX {
    uint32_t base;  // shared::cta address of the position array (same in every CTA)
    uint32_t shift;
};
__device__ __forceinline__ uint32_t vertex_addr(ClusterX c, uint32_t i) {
    return map_rank(c.base + ((i & ((1u << c.shift) - 1u)) << 4), i >> c.shift);
}
__device__ __forceinline__ float4 ldx(ClusterX c, uint32_t i) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(vertex_addr(c, i)));
    return v;
}
__device__ __forceinline__ void stx(ClusterX c, uint32_t i, float4 v) {
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(vertex_addr(c, i)), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w)
                 : "memory");
}


// Per-CTA partial results of UpdateSoftBodyState, read by rank 0 through distributed shared memory.
struct Partials {
    float val[12];  // min x, y, z | max x, y, z | predicted min x, y, z | predicted max x, y, z
    int idx[12];
    float sum[6];  // linear velocity, angular velocity sums
    int last_nan[6];  // last owned vertex with a NaN component (positions x, y, z, predicted x, y, z)
    float max_v_sq;   // largest squared vertex velocity before the clamp (the sleep test)
};

struct CShared {
    SCol cols[kMaxCollidingShapes];
    int ncols;
    int32_t table_slot;  // host-determined colliding shapes (-1: the context's colliders)
    int dynamic;         // some shape is a dynamic body
    uint32_t sensors;    // bit k: shape k is a sensor
    uint32_t sensor_hit;  // sensors touched by this CTA's vertices
    uint32_t ndyn;        // this CTA's owned vertices on dynamic shapes
    uint32_t dyn_updated;  // (rank 0) bit k: dynamic shape k took an impulse
    float dvel[kMaxCollidingShapes][6];  // (rank 0) the dynamic shapes' linear | angular velocities
    float six_volume;  // (rank 0) GetVolumeTimesSix of the substep
    int nan_flag[2];  // this CTA's vertices hold a NaN after the substep's integration (by substep parity)
    float delta[3];
    Partials part;
    int last_nan[6];  // over the whole body
    float red[32][4];
    int redi[32][4];
};

// Walks the dependency levels of one substep with every thread of the cluster. A level wider than one
// CTA is dealt round-robin over the cluster: thread g (= rank * T + tid) projects slots g, g + G, ...
// (G = cluster threads) and the level ends at a cluster barrier. A level of at most T slots goes to
// CTA 0 alone (slot s to thread s); a run of such levels is separated by CTA 0's own barriers and ends
// with one cluster barrier, which the other CTAs reach directly. Each thread loads its first record of
// the next level (and that level's descriptor) into registers before projecting the current one, so
// the load is in flight during the projection and the barrier; a thread's further slots of a level
// wider than the cluster are read where they are projected. No staging ring and no async-copy wait sit
// in the level's critical path.
template <int T, bool kGuard, bool kSkin>
__device__ __forceinline__ void cluster_levels(ClusterX cx, const BodyDesc &d, const uint4 *sdesc, uint32_t desc_cap, uint32_t rank,
                                               uint32_t G, float inv_dt_sq, SkinRefs sk) {
    const uint32_t L = d.num_levels;
    if (L == 0) return;
    const uint4 *__restrict__ rec = d.records;
    const uint4 *__restrict__ levels = d.levels;
    const uint32_t tid = threadIdx.x, g = rank * T + tid;
    auto desc = [&](uint32_t l) { return l < desc_cap ? sdesc[l] : __ldg(levels + l); };
    // First slot of this thread in a level of n slots (>= n: none) and the stride to its next slot.
    auto first_slot = [&](uint32_t n, uint32_t &stride) -> uint32_t {
        if (n <= uint32_t(T)) {
            stride = n;
            return rank == 0 ? tid : n;
        }
        stride = G;
        return g;
    };
    // This thread's first record of a level (a padding record when it has no slot there).
    auto first_record = [&](uint4 lv, uint32_t n) -> uint4 {
        uint32_t stride;
        const uint32_t s = first_slot(n, stride);
        return s < n ? __ldg(rec + lv.x + s) : make_uint4(0xffffffffu, 0u, 0u, 0u);
    };
    uint4 lv = desc(0);
    uint32_t end = desc(1).x;
    uint4 r0 = first_record(lv, end - lv.x);
    for (uint32_t l = 0; l < L; ++l) {
        const uint32_t n = end - lv.x;
        uint4 lv1 = lv, r1 = r0;
        uint32_t end1 = end;
        if (l + 1 < L) {  // the next level (sentinel descriptors follow the last level)
            lv1 = desc(l + 1);
            end1 = desc(l + 2).x;
            r1 = first_record(lv1, end1 - lv1.x);
        }
        uint32_t stride;
        uint32_t s = first_slot(n, stride);
        if (s < n) {
            if (r0.x != 0xffffffffu) project<kGuard>(cx, r0, slot_type(lv, s), inv_dt_sq, kSkin ? &sk : nullptr, false);
            for (s += stride; s < n; s += stride) {
                const uint4 r = __ldg(rec + lv.x + s);
                if (r.x != 0xffffffffu) project<kGuard>(cx, r, slot_type(lv, s), inv_dt_sq, kSkin ? &sk : nullptr, false);
            }
        }
        const bool narrow_pair = n <= uint32_t(T) && l + 1 < L && end1 - end <= uint32_t(T);
        if (narrow_pair) {
            if (rank == 0) __syncthreads();  // only CTA 0 works on both levels
        } else {
            cluster_barrier();
        }
        lv = lv1;
        end = end1;
        r0 = r1;
    }
}

// Dynamic shared memory of one CTA: positions [1 << shift] | level descriptors [desc_cap].
template <int T>
__global__ void __launch_bounds__(T) cluster_step_kernel(StepParams p, uint32_t shift, uint32_t desc_cap) {
    extern __shared__ float4 smem[];
    __shared__ CShared sh;
    const uint32_t tid = threadIdx.x;
    const uint32_t rank = cluster_rank(), C = cluster_size();
    const uint32_t item = blockIdx.x / C;  // one cluster per body
    if (item >= p.num_work) return;       // uniform over the cluster
    const uint32_t b = p.work[item];
    bool wake;
    if (!body_awake(p, b, wake)) return;  // asleep: not stepped (uniform over the cluster)
    const BodyDesc d = p.bodies[b];
    BodyState *st = p.states + b;
    const uint32_t nv = d.num_vertices;
    const uint32_t first = min(nv, rank << shift), last = min(nv, (rank + 1) << shift);
    float4 *sx = smem;
    uint4 *sdesc = reinterpret_cast<uint4 *>(smem + (size_t(1) << shift));
    const ClusterX cx{smem_u32(sx), shift};
    float4 *__restrict__ gx = p.x + d.vtx_offset;
    float4 *__restrict__ gv = p.v + d.vtx_offset;
    float4 *__restrict__ gprev = p.prev + d.vtx_offset;
    float4 *__restrict__ gplane = p.plane + d.vtx_offset;
    int32_t *__restrict__ gshape = p.shape + d.vtx_offset;

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

    // DetermineCollidingShapes, or the shapes the host determined for the body (every CTA evaluates it;
    // the result is the same), level descriptors and the positions this CTA owns.
    if (tid == 0) {
        const int32_t slot = p.table_slot ? p.table_slot[b] : -1;
        bool dynamic = false;
        const int n = slot >= 0 ? load_shape_table(p.tables + slot, sh.cols, dynamic) : colliding_shapes(p, d, st, body_pos, sh.cols);
        sh.ncols = n;
        sh.table_slot = slot;
        sh.dynamic = dynamic ? 1 : 0;
        sh.dyn_updated = 0;
        uint32_t sensors = 0;
        if (slot >= 0)
            for (int k = 0; k < n; ++k)
                if (sh.cols[k].flags & kColSensor) sensors |= 1u << k;
        sh.sensors = sensors;
        sh.sensor_hit = 0;
        if (dynamic)
            for (int k = 0; k < n; ++k)
                for (int j = 0; j < 3; ++j) {
                    sh.dvel[k][j] = p.tables[slot].e[k].lin[j];
                    sh.dvel[k][3 + j] = p.tables[slot].e[k].ang[j];
                }
    }
    const uint32_t nd = min(d.num_levels + 2, desc_cap);
    for (uint32_t l = tid; l < nd; l += T) sdesc[l] = __ldg(d.levels + l);
    for (uint32_t i = first + tid; i < last; i += T) sx[i - first] = gx[i];
    __syncthreads();

    // DetermineCollisionPlanes and DetermineSensorCollisions (owned vertices)
    const int ncols = sh.ncols;
    const bool has_dynamic = sh.dynamic != 0;  // (uniform over the cluster)
    const uint32_t sensors = sh.sensors;
    const HullRefs hr{p.hulls, p.hull_f4, p.hull_u32};
    uint32_t hits = 0;
    for (uint32_t i = first + tid; i < last; i += T) {
        const float4 pi = sx[i - first];
        int shape = -1;
        float4 plane = make_float4(0, 0, 0, 0);
        if (pi.w > 0.0f && ncols > 0) shape = collision_plane(xyz(pi), sh.cols, ncols, plane, hr);
        if (sensors && pi.w > 0.0f) hits |= sensor_hits(xyz(pi), sh.cols, ncols, sensors, hr);
        gshape[i] = shape;
        if (shape >= 0) gplane[i] = plane;
        if (p.contact) p.contact[d.vtx_offset + i] = 0;
    }
    if (hits) atomicOr(&sh.sensor_hit, hits);
    if (has_dynamic) {
        // The dynamic-body branch carries the body's velocities from one vertex to the next in index
        // order: each CTA lists its owned vertices on dynamic shapes (the shapes are fixed for the step);
        // rank 0 walks the lists in rank order, which is index order.
        __syncthreads();
        if (tid == 0) {
            int32_t *list = p.dyn_list + d.vtx_offset + first;
            uint32_t n = 0;
            for (uint32_t i = first; i < last; ++i) {
                const int s = gshape[i];
                if (s >= 0 && (sh.cols[s].flags & kColDynamic)) list[n++] = int32_t(i);
            }
            sh.ndyn = n;
        }
    }

    const float inv_dt_sq = 1.0f / (dt_sub * dt_sub);
    float damp = 1.0f - d.linear_damping * dt_sub;
    damp = damp < 0.0f ? 0.0f : damp;
    const f3 sub_g = g * dt_sub;
    const float nvf = float(nv > 0 ? nv : 1);
    const f3 sub_imp = (force * dt_sub) / nvf;
    const float restitution_threshold = -2.0f * len(g) * dt_sub;
    const uint32_t G = C * T;
    const uint32_t g0 = rank * T + tid;

    const bool has_pressure = d.pressure > 0.0f && d.num_faces > 0 && d.face_scratch;
    const bool skinned = d.skin_params && p.skin_ctl;
    const SkinCtl skin_ctl = skinned ? p.skin_ctl[b] : SkinCtl{};
    for (uint32_t it = 0; it < n_it; ++it) {
        // ApplyPressure (:291-323): per-face triple products dealt over the cluster into the body's face
        // scratch, their sum in face order by one thread (the reference sums sequentially), then per face
        // the impulse and per owned vertex its faces' impulses in face order.
        if (has_pressure) {
            float4 *fs = d.face_scratch;
            // every CTA's positions final (the staging, or the last substep's collision pass on the owned
            // vertices) before any face reads them
            cluster_barrier();
            for (uint32_t f = g0; f < d.num_faces; f += G) {
                const uint4 fc = __ldg(d.faces + f);
                fs[f] = make_float4(dot(cross(xyz(ldx(cx, fc.x)), xyz(ldx(cx, fc.y))), xyz(ldx(cx, fc.z))), 0.0f, 0.0f, 0.0f);
            }
            cluster_barrier();
            if (rank == 0 && tid == 0) {
                float six = 0.0f;
                for (uint32_t f = 0; f < d.num_faces; ++f) six = six + fs[f].x;
                sh.six_volume = six;
            }
            cluster_barrier();
            const float six = ld_cluster_f32(map_rank(smem_u32(&sh.six_volume), 0));
            if (six > 0.0f) {  // (the same value in every CTA)
                const float coefficient = jdiv(d.pressure * dt_sub, six);
                for (uint32_t f = g0; f < d.num_faces; f += G) {
                    const uint4 fc = __ldg(d.faces + f);
                    const f3 x1 = xyz(ldx(cx, fc.x)), x2 = xyz(ldx(cx, fc.y)), x3 = xyz(ldx(cx, fc.z));
                    fs[f] = with_w(coefficient * cross(x2 - x1, x3 - x1), 0.0f);
                }
                cluster_barrier();
                for (uint32_t i = first + tid; i < last; i += T) {
                    const float w = sx[i - first].w;
                    const float4 vel = gv[i];
                    f3 v = xyz(vel);
                    for (uint32_t k = __ldg(d.vf_off + i), ke = __ldg(d.vf_off + i + 1); k < ke; ++k) v = v + w * xyz(fs[__ldg(d.vf + k)]);
                    gv[i] = with_w(v, vel.w);
                }
            }
            cluster_barrier();  // every CTA has read the faces before they are written again
        }
        // IntegratePositions (owned vertices)
        bool nan_seen = false;
        for (uint32_t i = first + tid; i < last; i += T) {
            const float4 pi = sx[i - first];
            const float4 vel = gv[i];
            f3 v = xyz(vel);
            if (pi.w > 0.0f) {
                v = v + (sub_g + sub_imp * pi.w);
                v = v * damp;
            }
            gprev[i] = pi;
            gv[i] = with_w(v, vel.w);
            const f3 xn = xyz(pi) + v * dt_sub;
            nan_seen = nan_seen || has_nan(xn);
            sx[i - first] = with_w(xn, pi.w);
        }
        nan_seen = __syncthreads_or(nan_seen);
        if (tid == 0) sh.nan_flag[it & 1] = nan_seen ? 1 : 0;
        cluster_barrier();  // every position integrated before any constraint reads it
        if (it == 0 && wake && rank == 0 && tid == 0) p.sleep[b] = BodySleep{0.0f, 1u};  // (every CTA has read the record)
        // NaN-guarded projections when any CTA's vertices hold a NaN (flags double-buffered by substep)
        bool guard = false;
        for (uint32_t q = 0; q < C; ++q) guard = guard || ld_cluster_s32(map_rank(smem_u32(&sh.nan_flag[it & 1]), q)) != 0;
        // (skinned bodies get their own instantiation: the skin projection's registers stay out of the
        // common walk)
        if (skinned)
            cluster_levels<T, true, true>(cx, d, sdesc, desc_cap, rank, G, inv_dt_sq,
                                          SkinRefs{d.skin_params, d.skin_state, skin_ctl.max_distance_multiplier, skin_ctl.flags, n_it, it});
        else if (guard)
            cluster_levels<T, true, false>(cx, d, sdesc, desc_cap, rank, G, inv_dt_sq, SkinRefs{});
        else
            cluster_levels<T, false, false>(cx, d, sdesc, desc_cap, rank, G, inv_dt_sq, SkinRefs{});
        // ApplyCollisionConstraintsAndUpdateVelocities (owned vertices; the last level's barrier made
        // every remote write visible). The next integration touches owned vertices only.
        for (uint32_t i = first + tid; i < last; i += T) {
            const float4 pi = sx[i - first];
            if (!(pi.w > 0.0f)) continue;
            f3 x = xyz(pi);
            const float4 vel = gv[i];
            const float4 prev = gprev[i];
            const f3 prev_v = xyz(vel);
            f3 v = div3_rn(x - xyz(prev), dt_sub);
            const int shape = ncols > 0 ? gshape[i] : -1;
            if (has_dynamic && shape >= 0 && (sh.cols[shape].flags & kColDynamic)) continue;  // below, in vertex order
            if (shape >= 0 && collide_vertex(x, v, prev_v, gplane[i], sh.cols[shape], d.vertex_radius, dt_sub, restitution_threshold)) {
                sx[i - first] = with_w(x, pi.w);
                if (p.contact) p.contact[d.vtx_offset + i] = 1;
            }
            gv[i] = with_w(v, vel.w);
        }
        if (has_dynamic) {
            // The vertices on dynamic shapes, one thread of rank 0, in index order over the cluster (the
            // lists were complete at the integration's cluster barrier); the barrier after it makes the
            // remote position writes visible before the owners' next pass.
            if (rank == 0 && tid == 0) {
                const ShapeTable &tb = p.tables[sh.table_slot];
                for (uint32_t q = 0; q < C; ++q) {
                    const uint32_t nq = uint32_t(ld_cluster_s32(map_rank(smem_u32(&sh.ndyn), q)));
                    const int32_t *list = p.dyn_list + d.vtx_offset + min(nv, q << shift);
                    for (uint32_t k = 0; k < nq; ++k) {
                        const uint32_t i = uint32_t(list[k]);
                        const float4 pi = ldx(cx, i);
                        const float4 vel = gv[i];
                        const float4 prev = gprev[i];
                        const int s = gshape[i];
                        f3 x = xyz(pi), v = div3_rn(x - xyz(prev), dt_sub);
                        f3 lin = mk(sh.dvel[s][0], sh.dvel[s][1], sh.dvel[s][2]), ang = mk(sh.dvel[s][3], sh.dvel[s][4], sh.dvel[s][5]);
                        bool touched;
                        const bool impulse = collide_vertex_dynamic(x, v, xyz(vel), pi.w, gplane[i], tb.e[s], lin, ang, d.vertex_radius,
                                                                    dt_sub, restitution_threshold, touched);
                        if (touched && p.contact) p.contact[d.vtx_offset + i] = 1;
                        if (impulse) {
                            sh.dvel[s][0] = lin.x, sh.dvel[s][1] = lin.y, sh.dvel[s][2] = lin.z;
                            sh.dvel[s][3] = ang.x, sh.dvel[s][4] = ang.y, sh.dvel[s][5] = ang.z;
                            sh.dyn_updated |= 1u << s;
                        }
                        stx(cx, i, with_w(x, pi.w));
                        gv[i] = with_w(v, vel.w);
                    }
                }
            }
            cluster_barrier();
        }
    }

    // UpdateSoftBodyState: per-CTA partials over owned vertices, combined by rank 0.
    __syncthreads();
    const float max_sq = d.max_linear_velocity * d.max_linear_velocity;
    const int all[6] = {-1, -1, -1, -1, -1, -1};
    Bounds bd;
    bounds_init(bd);
    f3 lin = mk(0, 0, 0), ang = mk(0, 0, 0);
    bool finite = true;
    float max_v_sq = 0.0f;
    for (uint32_t i = first + tid; i < last; i += T) {
        const float4 pi = sx[i - first];
        f3 v = xyz(gv[i]), x = xyz(pi);
        const float vsq = len_sq(v);
        max_v_sq = fmaxf(max_v_sq, vsq);
        if (vsq > max_sq) v = v * jsqrt(jdiv(max_sq, vsq));
        gv[i] = with_w(v, 0.0f);
        lin = lin + v;
        ang = ang + cross(x, v);
        const f3 pred = (x + v * dt) + disp_g;
        bounds_add(bd, x, pred, int(i), all);
        finite = finite && isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
    }
    if (!finite) atomicOr(p.error, kErrNonFinite);
    bounds_reduce<T>(sh, bd);
    reduce_last_nan<T>(bd.last_nan, sh.last_nan);
    float sums[6];
    sums[0] = reduce_sum<T>(sh, lin.x, 0);
    sums[1] = reduce_sum<T>(sh, lin.y, 1);
    sums[2] = reduce_sum<T>(sh, lin.z, 2);
    sums[3] = reduce_sum<T>(sh, ang.x, 3);
    sums[4] = reduce_sum<T>(sh, ang.y, 0);
    sums[5] = reduce_sum<T>(sh, ang.z, 1);
    max_v_sq = reduce_max<T>(sh, max_v_sq, 2);
    auto write_bounds = [&]() {
        for (int k = 0; k < 3; ++k) {
            sh.part.val[k] = bd.mm[k], sh.part.idx[k] = bd.mi[k];
            sh.part.val[3 + k] = bd.xx[k], sh.part.idx[3 + k] = bd.xi[k];
            sh.part.val[6 + k] = bd.pm[k], sh.part.idx[6 + k] = bd.pmi[k];
            sh.part.val[9 + k] = bd.px[k], sh.part.idx[9 + k] = bd.pxi[k];
        }
    };
    if (tid == 0) {
        write_bounds();
        for (int k = 0; k < 6; ++k) sh.part.sum[k] = sums[k], sh.part.last_nan[k] = sh.last_nan[k];
        sh.part.max_v_sq = max_v_sq;
    }
    cluster_barrier();
    // The body's last NaN index per component (the maximum over the CTAs); a body holding NaNs repeats
    // its bounds over the vertices after it (the reference's sequential _mm_min_ps / _mm_max_ps).
    if (tid == 0) {
        int m[6] = {-1, -1, -1, -1, -1, -1};
        for (uint32_t q = 0; q < C; ++q) {
            const uint32_t base = map_rank(smem_u32(&sh.part), q) + uint32_t(offsetof(Partials, last_nan));
            for (int k = 0; k < 6; ++k) m[k] = max(m[k], ld_cluster_s32(base + 4u * k));
        }
        for (int k = 0; k < 6; ++k) sh.last_nan[k] = m[k];
    }
    __syncthreads();
    int skip[6];
    bool redo = false;
    for (int k = 0; k < 6; ++k) {
        skip[k] = sh.last_nan[k];
        redo = redo || skip[k] >= 0;
    }
    if (redo) {  // uniform over the cluster
        bounds_init(bd);
        for (uint32_t i = first + tid; i < last; i += T) {
            const f3 x = xyz(sx[i - first]), v = xyz(gv[i]);
            bounds_add(bd, x, (x + v * dt) + disp_g, int(i), skip);
        }
        bounds_reduce<T>(sh, bd);
        if (tid == 0) write_bounds();
        cluster_barrier();
    }
    if (rank == 0 && tid == 0) {
        Partials acc = sh.part;
        const uint32_t local = smem_u32(&sh.part);
        for (uint32_t r = 1; r < C; ++r) {
            const uint32_t base = map_rank(local, r);
            for (int k = 0; k < 12; ++k) {
                const float ov = ld_cluster_f32(base + uint32_t(offsetof(Partials, val)) + 4u * k);
                const int oi = ld_cluster_s32(base + uint32_t(offsetof(Partials, idx)) + 4u * k);
                if ((k / 3) & 1)
                    pick_max(acc.val[k], acc.idx[k], ov, oi);
                else
                    pick_min(acc.val[k], acc.idx[k], ov, oi);
            }
            for (int k = 0; k < 6; ++k) acc.sum[k] = acc.sum[k] + ld_cluster_f32(base + uint32_t(offsetof(Partials, sum)) + 4u * k);
            acc.max_v_sq = fmaxf(acc.max_v_sq, ld_cluster_f32(base + uint32_t(offsetof(Partials, max_v_sq))));
        }
        if (redo) {
            const float q = __int_as_float(0x7fffffff);
            for (int k = 0; k < 3; ++k) {
                if (skip[k] == int(nv) - 1) acc.val[k] = acc.val[3 + k] = q;
                if (skip[3 + k] == int(nv) - 1) acc.val[6 + k] = acc.val[9 + k] = q;
            }
        }
        const f3 delta = finish_body_state(st, d, body_pos, mk(acc.val[0], acc.val[1], acc.val[2]), mk(acc.val[3], acc.val[4], acc.val[5]),
                                           mk(acc.val[6], acc.val[7], acc.val[8]), mk(acc.val[9], acc.val[10], acc.val[11]), acc.sum,
                                           nvf);
        st3(sh.delta, delta);
        sleep_test(p, b, d, st, acc.max_v_sq);
        if (has_dynamic) {  // UpdateRigidBodyVelocities' inputs (:923-935) for the host
            ShapeTable &tb = p.tables[sh.table_slot];
            for (int k = 0; k < ncols; ++k)
                for (int j = 0; j < 3; ++j) {
                    tb.lin[k][j] = sh.dvel[k][j];
                    tb.ang[k][j] = sh.dvel[k][3 + j];
                }
            tb.updated = sh.dyn_updated;
        }
        if (p.sensor_contact) {  // the sensors touched by any CTA (the atomics precede the barriers since)
            uint32_t touched = sh.sensor_hit;
            for (uint32_t r = 1; r < C; ++r) touched |= uint32_t(ld_cluster_s32(map_rank(smem_u32(&sh.sensor_hit), r)));
            p.sensor_contact[b] = touched;
        }
    }
    cluster_barrier();
    f3 delta;
    {
        const uint32_t base = map_rank(smem_u32(sh.delta), 0);
        delta = mk(ld_cluster_f32(base), ld_cluster_f32(base + 4), ld_cluster_f32(base + 8));
    }
    const bool recentre = (d.flags & kFlagUpdatePosition) != 0;
    if (p.contact) {  // SoftBodyManifold: contact points before the recentring, and the offset
        for (uint32_t i = first + tid; i < last; i += T)
            if (p.contact[d.vtx_offset + i]) {
                const f3 x = xyz(sx[i - first]);
                const float4 pl = gplane[i];
                const f3 n = xyz(pl);
                p.contact_point[d.vtx_offset + i] = with_w(x - n * (dot(x, n) + pl.w), 0.0f);
            }
        if (rank == 0 && tid == 0) st3(p.contact_delta + 3 * size_t(b), recentre ? delta : mk(0.0f, 0.0f, 0.0f));
    }
    for (uint32_t i = first + tid; i < last; i += T) {
        const float4 pi = sx[i - first];
        gx[i] = recentre ? with_w(xyz(pi) - delta, pi.w) : pi;
    }
    if (d.skin_state) {  // the skin positions move with the body; SkinVertices has to run again
        if (recentre)
            for (uint32_t i = first + tid; i < last; i += T) {
                float4 &sp = d.skin_state[size_t(i) * 3 + 1];
                sp = with_w(xyz(sp) - delta, sp.w);
            }
        if (rank == 0 && tid == 0 && p.skin_ctl) p.skin_ctl[b].flags &= ~kSkinPreviousValid;
    }
    cluster_barrier();  // rank 0's shared memory stays alive until every CTA has read the offset
}

}  // namespace

// Bytes of dynamic shared memory of one cluster CTA.
size_t cluster_smem_bytes(uint32_t shift, uint32_t desc_cap) {
    return (size_t(1) << shift) * sizeof(float4) + size_t(desc_cap) * sizeof(uint4);
}

#define JSB_FOR_EACH_CLUSTER_SHAPE(X) X(128) X(256) X(512)

static cudaLaunchConfig_t cluster_config(int cluster, int threads, size_t smem, unsigned grid, cudaStream_t stream,
                                         cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, 1, 1);
    cfg.blockDim = dim3(unsigned(threads), 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    attr->id = cudaLaunchAttributeClusterDimension;
    attr->val.clusterDim.x = unsigned(cluster);
    attr->val.clusterDim.y = 1;
    attr->val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

// Launches one step of `p.num_work` bodies, one cluster of `cluster` CTAs each.
cudaError_t launch_cluster_step(const StepParams &p, int cluster, int threads, uint32_t shift, uint32_t desc_cap,
                                cudaStream_t stream) {
    cudaLaunchAttribute attr;
    const cudaLaunchConfig_t cfg = cluster_config(cluster, threads, cluster_smem_bytes(shift, desc_cap),
                                                  unsigned(cluster) * p.num_work, stream, &attr);
#define JSB_CLAUNCH(TT) \
    if (threads == TT) return cudaLaunchKernelEx(&cfg, cluster_step_kernel<TT>, p, shift, desc_cap);
    JSB_FOR_EACH_CLUSTER_SHAPE(JSB_CLAUNCH)
#undef JSB_CLAUNCH
    return cudaErrorInvalidValue;
}

// Allows the cluster kernels up to `max_dynamic_smem` bytes of dynamic shared memory and clusters of
// up to 16 CTAs (done once per device, outside any stream capture).
cudaError_t init_cluster_kernels(int max_dynamic_smem) {
    cudaError_t e = cudaSuccess;
#define JSB_CATTR(TT)                                                                                                        \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(cluster_step_kernel<TT>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                                   max_dynamic_smem);                                                       \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(cluster_step_kernel<TT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    JSB_FOR_EACH_CLUSTER_SHAPE(JSB_CATTR)
#undef JSB_CATTR
    return e;
}

// Clusters of this shape that fit on the device at once (0: the shape cannot be launched).
int cluster_occupancy(int cluster, int threads, size_t smem) {
    cudaLaunchAttribute attr;
    const cudaLaunchConfig_t cfg = cluster_config(cluster, threads, smem, unsigned(cluster), nullptr, &attr);
    int n = 0;
    cudaError_t e = cudaErrorInvalidValue;
#define JSB_COCC(TT) \
    if (threads == TT) e = cudaOccupancyMaxActiveClusters(&n, cluster_step_kernel<TT>, &cfg);
    JSB_FOR_EACH_CLUSTER_SHAPE(JSB_COCC)
#undef JSB_COCC
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace jsb
