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
#include "projection.cuh"

namespace jsb {
namespace {


struct Shared {
    SCol cols[kMaxCollidingShapes];
    SkinRefs skin;  // skinned bodies: written by thread 0 before each walk (no per-thread copy)
    int ncols;
    uint32_t item;
    float six_volume;
    float delta[3];
    uint64_t stage_bar;    // mbarrier of the bulk copies that stage a body's state (one phase per body)
    uint64_t ring_bar[2];  // mbarriers of the two halves of the schedule ring (one phase per chunk)
    int last_nan[6];
    float red[32][4];  // per-warp partials for reductions
    int redi[32][4];
    int32_t table_slot;  // host-determined colliding shapes of the body (-1: the context's colliders)
    int dynamic;         // a dynamic shape is among them
    uint32_t ndyn;       // vertices whose shape is dynamic (their list is in StepParams::dyn_list)
    uint32_t dyn_updated;
    float dvel[kMaxCollidingShapes][6];  // the dynamic shapes' velocities during the step
    uint32_t sensors;     // bit k: host-determined shape k belongs to a sensor
    uint32_t sensor_hit;  // bit k: a vertex penetrates sensor shape k (DetermineSensorCollisions)
};
static_assert(sizeof(Shared) + 256 <= 4096, "static shared memory of the solver kernels (the runtime reserves 4 KB)");


// ---- state staging: bulk copies on the TMA unit, completion on an mbarrier ----------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }

// Once per CTA, thread 0; the caller's barrier publishes it.
__device__ __forceinline__ void stage_bar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Thread 0: announces `bytes` for the barrier's current phase (its single arrival).
__device__ __forceinline__ void stage_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Thread 0: one bulk copy of `bytes` (a non-zero multiple of 16; both addresses 16-byte aligned) from
// global into shared memory, counted on `bar`.
__device__ __forceinline__ void stage_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// L2 eviction policies. The whole-step records of a batch stream through L2 once per step (hundreds of
// MB, more than L2 holds); copied with evict_first they do not push out the per-vertex collision planes,
// which are written at the start of the step and read again in every substep's collision pass, stored
// and loaded with evict_last.
__device__ __forceinline__ uint64_t l2_evict_first() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint64_t l2_evict_last() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// Thread 0: as stage_copy, for data read once (records and level descriptors of a schedule).
__device__ __forceinline__ void stage_copy_stream(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(l2_evict_first())
                 : "memory");
}

// A collision plane, kept in L2 (evict_last) between the writes at the start of a step and the reads of
// the substeps.
__device__ __forceinline__ void store_plane(float4 *dst, float4 v) {
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(dst), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w),
                 "l"(l2_evict_last())
                 : "memory");
}
__device__ __forceinline__ float4 load_plane(const float4 *src) {
    float4 v;
    asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(src), "l"(l2_evict_last())
                 : "memory");
    return v;
}

// Waits (bounded: about 2^20 polls) for phase `parity` of `bar`; false when it gave up.
__device__ __forceinline__ bool stage_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t it = 0; it < (1u << 20); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ---- schedule ring ----------------------------------------------------------------------------------
// A schedule's records and level descriptors reach shared memory chunk by chunk (host/schedule.h,
// build_stage_chunks): one thread issues two bulk copies per chunk (records, descriptors) on the TMA
// unit, completing on the mbarrier of one half of a two-half ring, two chunks ahead of the walk. A
// chunk is a run of levels that fits a half, so the walk's per-level critical path has no staging in
// it: descriptor and records from shared memory, positions from shared memory, projection, barrier.
struct StageRing {
    uint4 *rec;      // [2][half] record slots
    uint4 *desc;     // [2][kStageLevels + 1] level descriptors
    uint32_t half;   // record slots per half (>= the staged slots of every chunk of the bodies launched)
    uint64_t *bar;   // [2]
};

// Thread 0: stages chunk `ch` of a schedule into half h. The barrier that ended the walk's use of the
// half precedes this; the proxy fence orders those generic accesses before the copies.
__device__ __forceinline__ void ring_issue(const StageRing &ring, uint32_t h, uint4 ch, const uint4 *levels, const uint4 *records,
                                           uint32_t extra_desc) {
    const uint32_t rec_bytes = ch.w * uint32_t(sizeof(uint4));
    const uint32_t desc_bytes = (ch.y - ch.x + extra_desc) * uint32_t(sizeof(uint4));
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    stage_expect(&ring.bar[h], rec_bytes + desc_bytes);
    if (rec_bytes) stage_copy_stream(ring.rec + h * ring.half, records + ch.z, rec_bytes, &ring.bar[h]);
    stage_copy_stream(ring.desc + h * (kStageLevels + 1), levels + ch.x, desc_bytes, &ring.bar[h]);
}

// All threads: waits (bounded) for the chunk in half h. On a timeout the CTA reports it, gives the
// copies still in flight one more bounded wait, and must stop (returns false in every thread).
__device__ __forceinline__ bool ring_wait(const StageRing &ring, uint32_t h, uint32_t &phases, uint32_t num_pending, uint32_t *error) {
    const bool late = !stage_wait(&ring.bar[h], (phases >> h) & 1u);
    if (__syncthreads_or(late)) {
        if (threadIdx.x == 0) atomicOr(error, kErrTimeout);
        for (uint32_t k = 0; k < num_pending; ++k) stage_wait(&ring.bar[(h + k) & 1u], (phases >> ((h + k) & 1u)) & 1u);
        return false;
    }
    phases ^= 1u << h;
    return true;
}

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

// Walks the dependency levels of one substep's schedule (tape_cons: the taped forward's constraint
// inputs of this substep, 3 float4 per slot). Returns false when a staging wait gave up.
template <int T, bool kTape, bool kGuard>
__device__ __forceinline__ bool apply_levels(float4 *sx, const BodyDesc &d, float inv_dt_sq, const StageRing &ring,
                                             uint32_t &phases, float4 *tape_cons, uint32_t *error, const SkinRefs *sk) {
    const uint4 *__restrict__ levels = d.levels;
    const uint4 *__restrict__ rec = d.records;
    const uint4 *__restrict__ chunks = d.chunks;
    const uint32_t nc = d.num_chunks;
    if (nc == 0) return true;
    if (threadIdx.x == 0) {
        ring_issue(ring, 0, __ldg(chunks), levels, rec, 1);
        if (nc > 1) ring_issue(ring, 1, __ldg(chunks + 1), levels, rec, 1);
    }
    for (uint32_t c = 0; c < nc; ++c) {
        const uint32_t h = c & 1u;
        if (!ring_wait(ring, h, phases, nc - c < 2 ? nc - c : 2, error)) return false;
        const uint4 ch = __ldg(chunks + c);
        const uint4 *rr = ring.rec + h * ring.half;
        const uint4 *dd = ring.desc + h * (kStageLevels + 1);
        for (uint32_t l = 0; l < ch.y - ch.x; ++l) {
            const uint4 lv = dd[l];
            const uint32_t n = dd[l + 1].x - lv.x;
            const uint32_t rel = lv.x - ch.z;
            for (uint32_t s = threadIdx.x; s < n; s += T) {
                const uint4 r = rel + s < ch.w ? rr[rel + s] : __ldg(rec + lv.x + s);
                if (r.x != 0xffffffffu) {
                    if (kTape) tape_inputs(sx, r, slot_type(lv, s), tape_cons + size_t(lv.x + s) * 3);
                    project<kGuard>(sx, r, slot_type(lv, s), inv_dt_sq, sk, false);
                }
            }
            cta_sync<T>();
        }
        if (threadIdx.x == 0 && c + 2 < nc) ring_issue(ring, h, __ldg(chunks + c + 2), levels, rec, 1);
    }
    return true;
}

// ---------------------------------------------------------------------------------------------
// Whole-step walk (bodies without pressure): the constraint levels of every substep and, between them,
// each vertex's velocity update of the substep it leaves and integration of the substep it enters,
// placed by the host right after the vertex's own last constraint (csrc/host/schedule.h,
// build_step_schedule). Same reads and writes as the per-substep walk, so the same bits.
// ---------------------------------------------------------------------------------------------
struct VertexPass {
    float4 *sv, *sprev;  // shared memory (kSmemState)
    float4 *gv, *gprev;  // HBM (otherwise)
    const int32_t *gshape;
    const float4 *gplane;
    const SCol *cols;
    int ncols;
    f3 sub_g, sub_imp;
    float damp, dt_sub, radius, restitution_threshold;
    float4 *tape;  // taped forward: this step's substep states [substep][3][nv] (TapeDesc::state)
    uint32_t nv;
    uint8_t *contact;  // the body's contact flags (null: not recorded)
};

// ApplyCollisionConstraintsAndUpdateVelocities (:700-825, static colliders) of the substep vertex i
// leaves, then IntegratePositions (:325-365) of substep k it enters, for one vertex: the arithmetic of
// the two bulk passes of step_body in the same order. The taped forward step records the vertex's
// position after substep k - 1's constraints, and its position and velocity at the start of substep k,
// where the bulk passes of the per-substep walk record them.
template <bool kSmemState, bool kTape>
__device__ __forceinline__ void vertex_between_substeps(float4 *sx, const VertexPass &vp, uint32_t i, uint32_t k) {
    float4 pi = sx[i];
    float4 vel = kSmemState ? vp.sv[i] : vp.gv[i];
    if (kTape) vp.tape[(size_t(k - 1) * 3 + 2) * vp.nv + i] = pi;
    if (pi.w > 0.0f) {
        int shape = -1;
        float4 plane;
        if (vp.ncols > 0) {
            shape = kSmemState ? __float_as_int(vel.w) : vp.gshape[i];
            if (shape >= 0) plane = load_plane(vp.gplane + i);  // issued first: the longest latency of the pass
        }
        const float4 prev = kSmemState ? vp.sprev[i] : vp.gprev[i];
        f3 x = xyz(pi);
        const f3 prev_v = xyz(vel);
        f3 v = div3_rn(x - xyz(prev), vp.dt_sub);
        if (shape >= 0 && collide_vertex(x, v, prev_v, plane, vp.cols[shape], vp.radius, vp.dt_sub, vp.restitution_threshold)) {
            pi = with_w(x, pi.w);
            if (vp.contact) vp.contact[i] = 1;
        }
        v = v + (vp.sub_g + vp.sub_imp * pi.w);
        v = v * vp.damp;
        vel = with_w(v, vel.w);
    }
    if (kSmemState) {
        vp.sprev[i] = pi;
        vp.sv[i] = vel;
    } else {
        vp.gprev[i] = pi;
        vp.gv[i] = vel;
    }
    if (kTape) {
        vp.tape[size_t(k) * 3 * vp.nv + i] = pi;
        vp.tape[(size_t(k) * 3 + 1) * vp.nv + i] = with_w(xyz(vel), 0.0f);
    }
    sx[i] = with_w(xyz(pi) + xyz(vel) * vp.dt_sub, pi.w);
}

// Walks the whole-step schedule (tape_cons: the taped forward's constraint inputs of this step, 3 float4
// per whole-step slot). Returns false when a staging wait gave up.
template <int T, bool kSmemState, bool kGuard, bool kTape>
__device__ __forceinline__ bool apply_step_levels(float4 *sx, const BodyDesc &d, float inv_dt_sq, const StageRing &ring,
                                                  uint32_t &phases, const VertexPass &vp, float4 *tape_cons, uint32_t *error,
                                                  const SkinRefs *sk) {
    const uint4 *__restrict__ levels = d.step_levels;
    const uint4 *__restrict__ rec = d.step_records;
    const uint4 *__restrict__ chunks = d.step_chunks;
    const uint32_t nc = d.num_step_chunks;
    if (nc == 0) return true;
    if (threadIdx.x == 0) {
        ring_issue(ring, 0, __ldg(chunks), levels, rec, 0);
        if (nc > 1) ring_issue(ring, 1, __ldg(chunks + 1), levels, rec, 0);
    }
    for (uint32_t c = 0; c < nc; ++c) {
        const uint32_t h = c & 1u;
        if (!ring_wait(ring, h, phases, nc - c < 2 ? nc - c : 2, error)) return false;
        const uint4 ch = __ldg(chunks + c);
        const uint4 *rr = ring.rec + h * ring.half;
        const uint4 *dd = ring.desc + h * (kStageLevels + 1);
        for (uint32_t l = 0; l < ch.y - ch.x; ++l) {
            const uint4 lv = dd[l];
            const uint32_t rel = lv.x - ch.z;
            for (uint32_t s = threadIdx.x; s < lv.w; s += T) {
                const uint4 r = rel + s < ch.w ? rr[rel + s] : __ldg(rec + lv.x + s);
                if (r.x != 0xffffffffu) {
                    const int type = step_slot_type(lv, s);
                    if (type == 4) {
                        vertex_between_substeps<kSmemState, kTape>(sx, vp, r.x, r.y);
                    } else {
                        if (kTape) tape_inputs(sx, r, type, tape_cons + size_t(lv.x + s) * 3);
                        project<kGuard>(sx, r, type, inv_dt_sq, sk, true);
                    }
                }
            }
            cta_sync<T>();
        }
        if (threadIdx.x == 0 && c + 2 < nc) ring_issue(ring, h, __ldg(chunks + c + 2), levels, rec, 0);
    }
    return true;
}

// ---------------------------------------------------------------------------------------------
// One body, one step
// ---------------------------------------------------------------------------------------------
// Shared memory of one CTA (dynamic part), cap = the launch's largest vertex count:
//   kSmemState:  x[cap] | v[cap] (shape index in v.w) | prev[cap] | faces[...]
//   otherwise:   x[cap] | faces[...]       (v, prev, shape stay in HBM)
// faces: per-face triple product, then per-face pressure impulse (pressure bodies only).
// `phase`: parity of the staging barrier's current phase (flips once per body; the same in every thread);
// `ring_phases`: parities of the two schedule-ring halves (bit h; flip once per chunk).
// Returns false (in every thread) when a bounded wait for staged data gave up; the CTA must then stop.
template <int T, bool kSmemState, bool kTape = false>
__device__ bool step_body(const StepParams &p, uint32_t b, float4 *smem, uint32_t cap, Shared &sh, uint32_t &phase,
                          uint32_t &ring_phases) {
    const uint32_t tid = threadIdx.x;
    bool wake;
    if (!body_awake(p, b, wake)) return true;  // asleep: not stepped (uniform over the CTA)
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
    float4 *sface = smem + (kSmemState ? 3 * cap : cap);  // pressure faces; the schedule ring reuses it
    TapeDesc td = {};
    if (kTape) td = p.tape[b];
    StageRing ring;
    ring.rec = reinterpret_cast<uint4 *>(sface);
    ring.desc = ring.rec + 2 * p.ring_slots;
    ring.half = p.ring_slots;
    ring.bar = sh.ring_bar;

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

    // DetermineCollidingShapes: world AABB of (bounds U predicted bounds) grown by the vertex radius,
    // or the shapes the host determined for the body
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
        if (kTape)
            for (int k = 0; k < n; ++k)
                td.cols[size_t(p.tape_step) * kMaxCollidingShapes + k] = make_float2(sh.cols[k].friction, sh.cols[k].restitution);
    }
    // Stage the state in shared memory: one bulk copy per array (TMA unit), completing on the staging
    // barrier. The fence orders this CTA's earlier accesses of the destination (the previous body)
    // before the copies.
    if (tid == 0) {
        const uint32_t bytes = nv * uint32_t(sizeof(float4));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        stage_expect(&sh.stage_bar, kSmemState ? 2 * bytes : bytes);
        if (bytes > 0) {
            stage_copy(sx, gx, bytes, &sh.stage_bar);
            if (kSmemState) stage_copy(sv, gv, bytes, &sh.stage_bar);
        }
    }
    const bool timed_out = !stage_wait(&sh.stage_bar, phase);
    if (__syncthreads_or(timed_out)) {
        // Never expected. Report it, give the copies still in flight one more bounded wait so that none
        // lands in shared memory after the CTA has stopped, and stop this CTA's work: the body is left
        // as it was, and the results of the launch are not valid (jsb_synchronize returns
        // JSB_ERR_TIMEOUT).
        if (tid == 0) atomicOr(p.error, kErrTimeout);
        stage_wait(&sh.stage_bar, phase);
        return false;
    }
    phase ^= 1u;
    if (wake && tid == 0) p.sleep[b] = BodySleep{0.0f, 1u};  // (every thread has read the record)

    // DetermineCollisionPlanes (per vertex, once per step), and DetermineSensorCollisions
    const int ncols = sh.ncols;
    const bool has_dynamic = sh.dynamic != 0;
    const uint32_t sensors = sh.sensors;
    uint32_t hits = 0;
    for (uint32_t i = tid; i < nv; i += T) {
        float4 pi = sx[i];
        int shape = -1;
        float4 plane = make_float4(0, 0, 0, 0);
        if (pi.w > 0.0f && ncols > 0) shape = collision_plane(xyz(pi), sh.cols, ncols, plane, HullRefs{p.hulls, p.hull_f4, p.hull_u32});
        if (sensors && pi.w > 0.0f) hits |= sensor_hits(xyz(pi), sh.cols, ncols, sensors, HullRefs{p.hulls, p.hull_f4, p.hull_u32});
        if (kSmemState)
            sv[i].w = __int_as_float(shape);
        if (!kSmemState || p.contact) gshape[i] = shape;
        if (shape >= 0) store_plane(gplane + i, plane);
        if (p.contact) p.contact[d.vtx_offset + i] = 0;
        if (kTape) {
            td.plane[size_t(p.tape_step) * nv + i] = plane;
            td.shape[size_t(p.tape_step) * nv + i] = shape;
        }
    }
    if (hits) atomicOr(&sh.sensor_hit, hits);

    if (has_dynamic) {
        // The dynamic-body branch carries the body's velocities from one vertex to the next in index
        // order: list the vertices whose shape is dynamic (the shapes are fixed for the step).
        __syncthreads();
        if (tid == 0) {
            int32_t *list = p.dyn_list + d.vtx_offset;
            uint32_t n = 0;
            for (uint32_t i = 0; i < nv; ++i) {
                const int s = kSmemState ? __float_as_int(sv[i].w) : gshape[i];
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
    const bool has_pressure = d.pressure > 0.0f && d.num_faces > 0;
    // Whole-step walk: substep 0's integration below, then every substep's constraint levels with the
    // per-vertex passes between substeps inside the walk, then the last substep's velocity update.
    const bool step_walk = d.step_levels != nullptr && !has_pressure && !has_dynamic && (!kTape || td.step_slots > 0);
    VertexPass vp{};
    if (step_walk) {
        vp.sv = sv;
        vp.sprev = sprev;
        vp.gv = gv;
        vp.gprev = gprev;
        vp.gshape = gshape;
        vp.gplane = gplane;
        vp.cols = sh.cols;
        vp.ncols = ncols;
        vp.sub_g = sub_g;
        vp.sub_imp = sub_imp;
        vp.damp = damp;
        vp.dt_sub = dt_sub;
        vp.radius = d.vertex_radius;
        vp.restitution_threshold = restitution_threshold;
        vp.tape = kTape ? td.state + size_t(p.tape_step) * n_it * 3 * nv : nullptr;
        vp.nv = nv;
        vp.contact = p.contact ? p.contact + d.vtx_offset : nullptr;
    }
    const uint32_t passes = step_walk ? 1u : n_it;

    const SkinRefs *skin = d.skin_params && p.skin_ctl ? &sh.skin : nullptr;
    for (uint32_t it = 0; it < passes; ++it) {
        if (skin && tid == 0) {  // (read after the integration's barrier; the last walk ended at one)
            const SkinCtl ctl = p.skin_ctl[b];
            sh.skin = SkinRefs{d.skin_params, d.skin_state, ctl.max_distance_multiplier, ctl.flags, n_it, it};
        }
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
        bool nan_seen = false;
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
            const f3 xn = xyz(pi) + v * dt_sub;
            nan_seen = nan_seen || has_nan(xn);
            sx[i] = with_w(xn, pi.w);
            if (kTape) tape_state[nv + i] = with_w(v, 0.0f);
        }
        // Update groups in dependency-level order (NaN-guarded projections for a body holding NaNs)
        float4 *cons = kTape ? td.cons + (size_t(p.tape_step) * n_it + it) * size_t(td.slots) * 3 : nullptr;
        const bool nan_any = __syncthreads_or(nan_seen);
        bool walked;
        if (step_walk) {
            // (a body that turns non-finite within the step finishes it on the unguarded walk: same
            // result, slower)
            float4 *step_cons = kTape ? td.cons + size_t(p.tape_step) * td.step_slots * 3 : nullptr;
            if (nan_any)
                walked = apply_step_levels<T, kSmemState, true, kTape>(sx, d, inv_dt_sq, ring, ring_phases, vp, step_cons, p.error, skin);
            else
                walked = apply_step_levels<T, kSmemState, false, kTape>(sx, d, inv_dt_sq, ring, ring_phases, vp, step_cons, p.error, skin);
        } else if (nan_any)
            walked = apply_levels<T, kTape, true>(sx, d, inv_dt_sq, ring, ring_phases, cons, p.error, skin);
        else
            walked = apply_levels<T, kTape, false>(sx, d, inv_dt_sq, ring, ring_phases, cons, p.error, skin);
        if (!walked) return false;  // (uniform: decided at a barrier) the body is left half stepped, flagged
        __syncthreads();
        if (kTape) {  // position after the constraints of the last substep walked
            float4 *after = step_walk ? td.state + (size_t(p.tape_step) * n_it + n_it - 1) * 3 * nv : tape_state;
            for (uint32_t i = tid; i < nv; i += T) after[2 * nv + i] = sx[i];
        }
        // ApplyCollisionConstraintsAndUpdateVelocities (static colliders)
        for (uint32_t i = tid; i < nv; i += T) {
            float4 pi = sx[i];
            if (!(pi.w > 0.0f)) continue;
            f3 x = xyz(pi);
            float4 vel = kSmemState ? sv[i] : gv[i];
            float4 prev = kSmemState ? sprev[i] : gprev[i];
            f3 prev_v = xyz(vel);
            f3 v = div3_rn(x - xyz(prev), dt_sub);
            int shape = -1;
            if (ncols > 0) shape = kSmemState ? __float_as_int(vel.w) : gshape[i];
            if (has_dynamic && shape >= 0 && (sh.cols[shape].flags & kColDynamic)) continue;  // below, in vertex order
            if (shape >= 0 && collide_vertex(x, v, prev_v, load_plane(gplane + i), sh.cols[shape], d.vertex_radius, dt_sub, restitution_threshold)) {
                sx[i] = with_w(x, pi.w);
                if (p.contact) p.contact[d.vtx_offset + i] = 1;
            }
            if (kSmemState)
                sv[i] = with_w(v, vel.w);
            else
                gv[i] = with_w(v, vel.w);
        }
        __syncthreads();
        if (has_dynamic) {  // the vertices on dynamic shapes, one thread, in index order
            if (tid == 0) {
                const ShapeTable &tb = p.tables[sh.table_slot];
                const int32_t *list = p.dyn_list + d.vtx_offset;
                for (uint32_t k = 0; k < sh.ndyn; ++k) {
                    const uint32_t i = uint32_t(list[k]);
                    const float4 pi = sx[i];
                    const float4 vel = kSmemState ? sv[i] : gv[i];
                    const float4 prev = kSmemState ? sprev[i] : gprev[i];
                    const int s = kSmemState ? __float_as_int(vel.w) : gshape[i];
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
                    sx[i] = with_w(x, pi.w);
                    if (kSmemState)
                        sv[i] = with_w(v, vel.w);
                    else
                        gv[i] = with_w(v, vel.w);
                }
            }
            __syncthreads();
        }
    }

    // UpdateSoftBodyState
    const float max_sq = d.max_linear_velocity * d.max_linear_velocity;
    const int all[6] = {-1, -1, -1, -1, -1, -1};
    Bounds bd;
    bounds_init(bd);
    f3 lin = mk(0, 0, 0), ang = mk(0, 0, 0);
    bool finite = true;
    float max_v_sq = 0.0f;
    for (uint32_t i = tid; i < nv; i += T) {
        float4 pi = sx[i];
        float4 vel = kSmemState ? sv[i] : gv[i];
        f3 v = xyz(vel), x = xyz(pi);
        float vsq = len_sq(v);
        max_v_sq = fmaxf(max_v_sq, vsq);
        if (vsq > max_sq) v = v * jsqrt(jdiv(max_sq, vsq));
        gv[i] = with_w(v, 0.0f);
        lin = lin + v;
        ang = ang + cross(x, v);
        f3 pred = (x + v * dt) + disp_g;
        bounds_add(bd, x, pred, int(i), all);
        finite = finite && isfinite(x.x) && isfinite(x.y) && isfinite(x.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z);
    }
    if (!finite) atomicOr(p.error, kErrNonFinite);
    if (__syncthreads_or(!finite)) {
        // NaN components: extremes over the vertices after the last NaN (the reference's sequential
        // _mm_min_ps / _mm_max_ps semantics)
        reduce_last_nan<T>(bd.last_nan, sh.last_nan);
        int skip[6];
        for (int k = 0; k < 6; ++k) skip[k] = sh.last_nan[k];
        bounds_init(bd);
        for (uint32_t i = tid; i < nv; i += T) {
            const f3 x = xyz(sx[i]), v = xyz(gv[i]);
            bounds_add(bd, x, (x + v * dt) + disp_g, int(i), skip);
        }
        bounds_reduce<T>(sh, bd);
        bounds_nan_tail(bd, skip, int(nv));
    } else {
        bounds_reduce<T>(sh, bd);
    }
    float sums[6];
    sums[0] = reduce_sum<T>(sh, lin.x, 0);
    sums[1] = reduce_sum<T>(sh, lin.y, 1);
    sums[2] = reduce_sum<T>(sh, lin.z, 2);
    sums[3] = reduce_sum<T>(sh, ang.x, 3);
    sums[4] = reduce_sum<T>(sh, ang.y, 0);
    sums[5] = reduce_sum<T>(sh, ang.z, 1);
    max_v_sq = reduce_max<T>(sh, max_v_sq, 2);
    if (tid == 0) {
        const f3 delta = finish_body_state(st, d, body_pos, mk(bd.mm[0], bd.mm[1], bd.mm[2]), mk(bd.xx[0], bd.xx[1], bd.xx[2]),
                                           mk(bd.pm[0], bd.pm[1], bd.pm[2]), mk(bd.px[0], bd.px[1], bd.px[2]), sums, nvf);
        st3(sh.delta, delta);
        sleep_test(p, b, d, st, max_v_sq);
        if (has_dynamic) {  // UpdateRigidBodyVelocities' inputs (:923-935) for the host
            ShapeTable &tb = p.tables[sh.table_slot];
            for (int k = 0; k < ncols; ++k)
                for (int j = 0; j < 3; ++j) {
                    tb.lin[k][j] = sh.dvel[k][j];
                    tb.ang[k][j] = sh.dvel[k][3 + j];
                }
            tb.updated = sh.dyn_updated;
        }
    }
    __syncthreads();
    const f3 delta = ld3(sh.delta);
    const bool shift = (d.flags & kFlagUpdatePosition) != 0;
    if (p.contact) {  // SoftBodyManifold (read by OnSoftBodyContactAdded before the recentring): contact points
        for (uint32_t i = tid; i < nv; i += T)
            if (p.contact[d.vtx_offset + i]) {
                const f3 x = xyz(sx[i]);
                const float4 pl = gplane[i];
                const f3 n = xyz(pl);
                p.contact_point[d.vtx_offset + i] = with_w(x - n * (dot(x, n) + pl.w), 0.0f);
            }
        if (tid == 0) st3(p.contact_delta + 3 * size_t(b), shift ? delta : mk(0.0f, 0.0f, 0.0f));
    }
    if (tid == 0 && p.sensor_contact) p.sensor_contact[b] = sh.sensor_hit;  // (barriers since the atomics)
    for (uint32_t i = tid; i < nv; i += T) {
        float4 pi = sx[i];
        gx[i] = shift ? with_w(xyz(pi) - delta, pi.w) : pi;
    }
    if (d.skin_state) {  // UpdateSoftBodyState (:889-892, :916-917): the skin positions move with the body
        if (shift)
            for (uint32_t i = tid; i < nv; i += T) {
                float4 &sp = d.skin_state[size_t(i) * 3 + 1];
                sp = with_w(xyz(sp) - delta, sp.w);
            }
        if (tid == 0 && p.skin_ctl) p.skin_ctl[b].flags &= ~kSkinPreviousValid;
    }
    __syncthreads();
    return true;
}

template <int T, bool kSmemState, bool kTape>
__device__ __forceinline__ void step_queue(const StepParams &p, uint32_t cap, float4 *smem, Shared &sh) {
    if (threadIdx.x == 0) {
        stage_bar_init(&sh.stage_bar);
        stage_bar_init(&sh.ring_bar[0]);
        stage_bar_init(&sh.ring_bar[1]);
    }
    uint32_t phase = 0, ring_phases = 0;
    for (;;) {
        if (threadIdx.x == 0) sh.item = atomicAdd(p.queue, 1u);
        __syncthreads();
        const uint32_t item = sh.item;
        __syncthreads();
        if (item >= p.num_work) return;
        if (!step_body<T, kSmemState, kTape>(p, p.work[item], smem, cap, sh, phase, ring_phases)) return;
    }
}

// Register budget of 128 per thread (65,536 / (T x 512 / T)): enough for the projections without
// spilling, and small CTAs of small bodies still pack many to an SM.
template <int T, bool kSmemState>
__global__ void __launch_bounds__(T, 512 / T) step_kernel(StepParams p, uint32_t cap) {
    extern __shared__ float4 smem[];
    __shared__ Shared sh;
    step_queue<T, kSmemState, false>(p, cap, smem, sh);
}

// The taped forward step (differentiable runs) holds more live values; one CTA per SM lets it keep
// them in registers.
template <int T, bool kSmemState>
__global__ void __launch_bounds__(T, 1) step_kernel_tape(StepParams p, uint32_t cap) {
    extern __shared__ float4 smem[];
    __shared__ Shared sh;
    step_queue<T, kSmemState, true>(p, cap, smem, sh);
}

}  // namespace

// Bytes of dynamic shared memory for a launch whose largest body has `vertices` vertices and whose
// largest pressurised body has `faces` faces.
size_t step_smem_bytes(bool smem_state, uint32_t vertices, uint32_t faces, uint32_t ring_slots) {
    const size_t faces_bytes = size_t(faces) * sizeof(float4);
    const size_t ring_bytes = (2 * size_t(ring_slots) + 2 * (kStageLevels + 1)) * sizeof(uint4);
    return size_t(vertices) * sizeof(float4) * (smem_state ? 3 : 1) + (faces_bytes > ring_bytes ? faces_bytes : ring_bytes);
}

#define JSB_FOR_EACH_SHAPE(X) \
    X(32, true) X(64, true) X(128, true) X(256, true) X(512, true) X(32, false) X(64, false) X(128, false) X(256, false) X(512, false)

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

#define JSB_FOR_EACH_TAPE_SHAPE(X) X(128, true) X(256, true) X(128, false) X(256, false)

// Taped forward step (differentiable runs): 128 or 256 threads per CTA, every body of the launch.
cudaError_t launch_step_tape(const StepParams &p, int threads, bool smem_state, uint32_t smem_vertices, uint32_t smem_faces, int grid,
                             cudaStream_t stream) {
    size_t smem = step_smem_bytes(smem_state, smem_vertices, smem_faces, p.ring_slots);
#define JSB_LAUNCH_TAPE(TT, SS)                                                   \
    if (threads == TT && smem_state == SS) {                                      \
        step_kernel_tape<TT, SS><<<grid, TT, smem, stream>>>(p, smem_vertices);   \
        return cudaGetLastError();                                                \
    }
    JSB_FOR_EACH_TAPE_SHAPE(JSB_LAUNCH_TAPE)
#undef JSB_LAUNCH_TAPE
    return cudaErrorInvalidValue;
}

int step_tape_occupancy(int threads, bool smem_state, size_t smem) {
    int n = 0;
#define JSB_OCC_TAPE(TT, SS) \
    if (threads == TT && smem_state == SS) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel_tape<TT, SS>, TT, smem);
    JSB_FOR_EACH_TAPE_SHAPE(JSB_OCC_TAPE)
#undef JSB_OCC_TAPE
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
#define JSB_ATTR_TAPE(TT, SS) \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(step_kernel_tape<TT, SS>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem);
    JSB_FOR_EACH_TAPE_SHAPE(JSB_ATTR_TAPE)
#undef JSB_ATTR_TAPE
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
constexpr size_t kOffChunks = kOffVf + (3 * kMaxFaces) / 4;        // uint4[kMaxLevels] staging chunks
constexpr size_t kScratchFloat4 = kOffChunks + kMaxLevels;         // about 2.4 MB
constexpr uint32_t kRingHalf = 256;                                // schedule-ring half, record slots

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
    p.ring_slots = kRingHalf;
    p.sleep = nullptr;  // (bodies that may sleep are refused by jsb_step_body_noalloc)
    p.tables = nullptr;
    p.table_slot = nullptr;
    p.dyn_list = nullptr;
    p.hulls = nullptr;
    p.hull_f4 = nullptr;
    p.hull_u32 = nullptr;
    p.contact = nullptr;
    p.contact_point = nullptr;
    p.contact_delta = nullptr;
    p.sensor_contact = nullptr;
    p.skin_ctl = nullptr;
    if (threadIdx.x == 0) {
        stage_bar_init(&sh.stage_bar);
        stage_bar_init(&sh.ring_bar[0]);
        stage_bar_init(&sh.ring_bar[1]);
    }
    __syncthreads();
    uint32_t phase = 0, ring_phases = 0;
    step_body<T, kSmemState>(p, 0, smem, cap, sh, phase, ring_phases);
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
    if (creation->allow_sleeping)
        return report_error(JSB_ERR_UNSUPPORTED, "jsb_step_body_noalloc keeps no sleep state: create the body with "
                                                 "allow_sleeping = 0, or step it in a context");
    if (num_colliders > kMaxColliders)
        return report_error(JSB_ERR_CAPACITY, "jsb_step_body_noalloc takes at most " + std::to_string(kMaxColliders) + " colliders");
    for (uint32_t i = 0; i < num_colliders; ++i)
        if (colliders[i].type < JSB_COLLIDER_BOX || colliders[i].type > JSB_COLLIDER_CYLINDER)
            return report_error(JSB_ERR_INVALID_ARGUMENT, "unknown collider type");

    // Host side: parse the settings and build the padded dependency-level schedule.
    ParsedSettings ps;
    bool unsupported = false;
    std::string err = parse_settings(settings_blob, len, ps, unsupported);
    if (!err.empty()) return report_error(unsupported ? JSB_ERR_UNSUPPORTED : JSB_ERR_BLOB, err);
    if (!ps.skinned.empty()) return report_error(JSB_ERR_UNSUPPORTED, "jsb_step_body_noalloc does not take skinned constraints");
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
    const std::vector<uint32_t> chunks = build_stage_chunks(sched.padded_levels, sched.num_levels, true, kRingHalf);
    e = copy(kOffLevels, sched.padded_levels.data(), sched.padded_levels.size() * sizeof(uint32_t));
    if (e == cudaSuccess) e = copy(kOffChunks, chunks.data(), chunks.size() * sizeof(uint32_t));
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
    d.chunks = reinterpret_cast<const uint4 *>(scratch + kOffChunks);
    d.num_chunks = uint32_t(chunks.size() / 4);
    d.stage_half = kRingHalf;
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
    const uint32_t ring_slots = kRingHalf;
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
