// C ABI of the GPU soft-body solver (include/jsb.h): contexts, settings upload, bodies, stepping,
// readback, CUDA graphs and the per-bucket launch-shape autotuner.
//
// Host-side flow for one step of all bodies (jsb_step):
//   1. upload pending AddForce accumulators (one copy) when any body has one;
//   2. zero the per-bucket work-queue counters;
//   3. fork: one persistent launch of the solver kernel per body-size bucket, each on its own stream
//      (buckets differ in threads per CTA and dynamic shared memory), joined back on the caller's stream;
//   4. clear the device force array if it was non-zero.
// The same sequence is recorded into a CUDA graph by jsb_step_graph.

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../../include/jsb.h"
#include "../kernels/device_types.h"
#include "schedule.h"

namespace jsb {

cudaError_t launch_step(const StepParams &p, int threads, bool smem_state, uint32_t smem_vertices, uint32_t smem_faces,
                        int grid, cudaStream_t stream);
int step_occupancy(int threads, bool smem_state, size_t smem);
size_t step_smem_bytes(bool smem_state, uint32_t vertices, uint32_t faces, uint32_t ring_slots);
cudaError_t init_step_kernels(int max_dynamic_smem);
cudaError_t launch_step_tape(const StepParams &p, int threads, bool smem_state, uint32_t smem_vertices, uint32_t smem_faces, int grid,
                             cudaStream_t stream);
int step_tape_occupancy(int threads, bool smem_state, size_t smem);
size_t cluster_smem_bytes(uint32_t shift, uint32_t desc_cap);
cudaError_t launch_cluster_step(const StepParams &p, int cluster, int threads, uint32_t shift, uint32_t desc_cap,
                                cudaStream_t stream);
cudaError_t init_cluster_kernels(int max_dynamic_smem);
int cluster_occupancy(int cluster, int threads, size_t smem);
size_t adjoint_smem_bytes(uint32_t vertices, uint32_t faces, uint32_t depth, uint32_t rpt, int threads);
cudaError_t init_adjoint_kernels(int max_dynamic_smem);
int adjoint_occupancy(size_t smem, int threads);
cudaError_t launch_adjoint(const AdjParams &q, uint32_t cap_vertices, uint32_t cap_faces, int grid, int threads, cudaStream_t stream);
cudaError_t launch_add(float4 *dst, const float4 *src, uint64_t n, int num_sms, cudaStream_t stream);
cudaError_t launch_unpack_state(const float *pos3, const float *vel3, float4 *x, float4 *v, uint64_t n, int num_sms,
                                cudaStream_t stream);
cudaError_t launch_pack_state(const float4 *x, const float4 *v, float *pos3, float *vel3, uint64_t n, int num_sms,
                              cudaStream_t stream);

namespace {

thread_local std::string g_last_error;

jsb_status fail(jsb_status code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define JSB_CUDA(call)                                                                                      \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess)                                                                              \
            return fail(e_ == cudaErrorMemoryAllocation ? JSB_ERR_OUT_OF_MEMORY : JSB_ERR_CUDA,              \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                                \
    } while (0)

template <class T>
struct DevBuf {
    T *ptr = nullptr;
    size_t count = 0;     // elements in use
    size_t capacity = 0;  // elements allocated
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : ptr(o.ptr), count(o.count), capacity(o.capacity) {
        o.ptr = nullptr;
        o.count = o.capacity = 0;
    }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) {
            reset();
            ptr = o.ptr;
            count = o.count;
            capacity = o.capacity;
            o.ptr = nullptr;
            o.count = o.capacity = 0;
        }
        return *this;
    }
    ~DevBuf() { reset(); }
    void reset() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = capacity = 0;
    }
    cudaError_t alloc(size_t n) {
        reset();
        if (n == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&ptr, n * sizeof(T));
        if (e == cudaSuccess) count = capacity = n;
        return e;
    }
    // Keeps the allocation when it is large enough (contents undefined), else allocates anew.
    cudaError_t ensure(size_t n) {
        if (ptr && n <= capacity) {
            count = n;
            return cudaSuccess;
        }
        return alloc(n);
    }
    cudaError_t upload(const T *src, size_t n) {
        cudaError_t e = alloc(n);
        if (e != cudaSuccess || n == 0) return e;
        return cudaMemcpy(ptr, src, n * sizeof(T), cudaMemcpyHostToDevice);
    }
};

// Whole-step schedule of one settings object for one iteration count (bodies without pressure).
struct StepSchedRec {
    StepSchedule sched;
    DevBuf<uint4> levels, records;
    std::map<uint32_t, std::pair<DevBuf<uint4>, uint32_t>> chunks;  // staging chunks by ring half: (table, count)
};

struct SettingsRec {
    ParsedSettings parsed;
    Schedule schedule;
    std::vector<uint32_t> vf_off, vf;
    DevBuf<uint4> levels, records, faces;
    DevBuf<uint32_t> vf_off_dev, vf_dev;
    DevBuf<float4> skin_params;  // per skinned constraint {max distance, back stop distance, back stop radius, vertex}
    std::map<uint32_t, std::unique_ptr<StepSchedRec>> steps;  // by iteration count; null: none (a level too wide)
    std::map<uint32_t, std::pair<DevBuf<uint4>, uint32_t>> chunks;  // staging chunks of `schedule` by ring half
};

struct BodyRec {
    uint32_t settings_id;
    jsb_creation_settings creation;
    BodyState state;  // host copy, authoritative until the first upload
    uint32_t vtx_offset = 0;
};

// Bodies are bucketed by vertex count; each bucket is one persistent launch per step with its own
// threads per CTA and vertex-state placement, chosen by the autotuner.
struct Bucket {
    uint32_t max_vertices;
    int threads;
    int state_mode;  // 0: x, v, prev in shared memory when they fit; 1: only positions in shared memory;
                     // 2: thread-block-cluster path
};

struct LaunchGroup {  // the bodies of one bucket (or every body on the cluster path)
    int cluster = 0;  // > 0: CTAs per cluster, one cluster per body (cluster.cu)
    uint32_t shift = 0, desc_cap = 0;  // cluster path: vertices per CTA (log2), cached level descriptors
    int threads = 0;
    bool smem_state = true;  // velocities / previous positions staged in shared memory
    uint32_t smem_vertices = 0, smem_faces = 0;
    uint32_t ring_slots = 32;  // record slots per schedule-ring half (staging chunks are built for it)
    int grid = 0;
    std::vector<uint32_t> bodies;
    DevBuf<uint32_t> work;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

// The bodies of one launch group in a differentiable run, with the taped-forward and adjoint launch
// shapes sized for them (the groups run concurrently on their own streams, like the forward step).
struct AdjGroup {
    DevBuf<uint32_t> work;
    uint32_t num_work = 0;
    uint32_t cap_vertices = 0, cap_faces = 0, ring_slots = 32, max_level_slots = 0;  // ring_slots: the forward group's
    int threads = 128;  // taped forward and adjoint CTAs: 256 when levels are wider than 192 slots
    bool tape_smem_state = true;
    int tape_grid = 1, adj_grid = 1;
    uint32_t adj_depth = 0, adj_rpt = 1;  // adjoint record / tape ring: levels ahead, slots per thread
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
};

// State of one differentiable run (jsb_adjoint_*): checkpoints every `every` steps, the tape of one
// checkpoint segment, adjoint accumulators and loss seeds.
struct AdjointSession {
    ~AdjointSession() { release_launch_groups(); }
    void release_launch_groups() {
        for (AdjGroup &g : groups) {
            if (g.stream) cudaStreamDestroy(g.stream);
            if (g.done) cudaEventDestroy(g.done);
        }
        groups.clear();
        if (fork) cudaEventDestroy(fork);
        fork = nullptr;
    }
    std::vector<AdjGroup> groups;
    cudaEvent_t fork = nullptr;
    float dt = 0.0f;
    int steps = 0, every = 1;
    bool forward_done = false, backward_done = false;
    int cur_step = 0;  // steps run by jsb_adjoint_forward so far
    std::vector<DevBuf<float4>> ckpt_x, ckpt_v;
    std::vector<DevBuf<BodyState>> ckpt_state;
    DevBuf<float4> final_x, final_v;
    DevBuf<BodyState> final_state;
    DevBuf<float4> tape_cons, tape_state, tape_plane;
    DevBuf<int32_t> tape_shape;
    DevBuf<float2> tape_cols;
    DevBuf<float> grad_slots, grad_force;
    DevBuf<TapeDesc> tape_desc;
    std::vector<size_t> slot_offset;  // per body, into grad_slots
    std::vector<uint32_t> step_slots;  // per body: slots of the whole-step schedule it walks, 0 = per-substep walk
    DevBuf<float4> adj_x, adj_v, seed_dev;
    std::vector<std::pair<int, std::vector<float4>>> seeds;  // (step, dL/dx of every vertex)
    int tape_segment = -1;  // checkpoint segment whose tape is in the tape buffers
    float forward_ms = 0.0f, recompute_ms = 0.0f, reverse_ms = 0.0f;  // device time of the last run's phases
};

// Device time between events recorded on the legacy default stream (the phases' fork / join stream).
struct PhaseTimer {
    std::vector<cudaEvent_t> ev;
    cudaError_t mark() {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        ev.push_back(e);
        return cudaEventRecord(e, 0);
    }
    float between(size_t a, size_t b) const {
        float ms = 0.0f;
        return cudaEventElapsedTime(&ms, ev[a], ev[b]) == cudaSuccess ? ms : 0.0f;
    }
    ~PhaseTimer() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
};

}  // namespace

// Lets other translation units of the library report failures through jsb_last_error_string.
jsb_status report_error(jsb_status code, const std::string &msg) { return fail(code, msg); }

}  // namespace jsb

struct jsb_context {
    int device = 0;
    int num_sms = 0;
    size_t max_smem_optin = 0;
    float gravity[3] = {0.0f, -9.81f, 0.0f};
    std::vector<std::unique_ptr<jsb::SettingsRec>> settings;
    std::vector<jsb::BodyRec> bodies;
    std::vector<jsb::ColliderDev> colliders;
    std::vector<jsb::Bucket> buckets;
    int cluster_size = 0;       // CTAs per cluster on the cluster path, 0 = largest that fits
    int cluster_threads = 256;  // threads per CTA on the cluster path
    bool step_walk = true;  // walk whole-step schedules where a body has one (jsb_set_step_walk)
    // device state
    bool dirty = true;  // structure changed: device arrays must be rebuilt
    bool groups_dirty = true;  // bucket table changed: launch groups must be rebuilt
    uint64_t total_vertices = 0;
    jsb::DevBuf<float4> x, v, prev, plane;
    jsb::DevBuf<int32_t> shape;
    jsb::DevBuf<jsb::BodyDesc> descs;
    std::vector<jsb::BodyDesc> descs_host;  // staging chunks are set when the launch groups are built
    jsb::DevBuf<jsb::BodyState> states;
    jsb::DevBuf<jsb::ColliderDev> colliders_dev;
    jsb::DevBuf<uint32_t> queues;
    jsb::DevBuf<uint32_t> error;
    jsb::DevBuf<float> forces;  // per body: 3 floats consumed by the next step
    jsb::DevBuf<float> step_forces;  // per body: 3 floats applied before every step
    jsb::DevBuf<jsb::BodySleep> sleep;  // per body: sleep timer, active flag
    std::map<uint32_t, std::vector<jsb::ShapeEntry>> table_host;  // host-determined colliding shapes by body
    std::vector<jsb::HullDev> hulls_host;  // registered convex hulls (jsb_hull_add) and their data
    std::vector<float4> hull_f4_host;
    std::vector<uint32_t> hull_u32_host;
    bool hulls_dirty = false;
    bool contact_readback = false;  // record SoftBodyManifold data every step (jsb_set_contact_readback)
    jsb::DevBuf<uint8_t> contact;
    jsb::DevBuf<float4> contact_point;
    jsb::DevBuf<float> contact_delta;
    jsb::DevBuf<uint32_t> sensor_contact;  // per body: sensor shapes of its table with a vertex inside
    jsb::DevBuf<float4> skin_state;        // 3 per vertex (SkinState) when any body has skinned constraints
    jsb::DevBuf<jsb::SkinCtl> skin_ctl;    // per body
    jsb::DevBuf<float4> face_scratch;      // pressure bodies: one float4 per face (cluster path)
    std::vector<size_t> face_off;          // per body, into face_scratch
    jsb::DevBuf<jsb::HullDev> hulls_dev;
    jsb::DevBuf<float4> hull_f4_dev;
    jsb::DevBuf<uint32_t> hull_u32_dev;
    bool tables_dirty = false;
    std::vector<int32_t> table_slot_host;
    std::vector<jsb::ShapeTable> tables_staging;
    jsb::DevBuf<jsb::ShapeTable> tables_dev;
    jsb::DevBuf<int32_t> table_slot_dev;
    jsb::DevBuf<int32_t> dyn_list;
    float sleep_velocity_threshold = 0.03f;  // PhysicsSettings::mPointVelocitySleepThreshold (PhysicsSettings.h:102)
    float time_before_sleep = 0.5f;          // PhysicsSettings::mTimeBeforeSleep (PhysicsSettings.h:95)
    std::vector<float> step_force_host;
    jsb::DevBuf<float> staging3;  // host round trip: positions then velocities, 3 floats per vertex
    std::vector<float> pending_force;
    float *pending_force_pinned = nullptr;
    bool forces_pending = false;
    std::vector<jsb::LaunchGroup> groups;
    std::vector<uint32_t> single_work_host;
    jsb::DevBuf<uint32_t> single_work;  // identity list for the plain form
    std::unique_ptr<jsb::AdjointSession> adjoint;
    std::unique_ptr<jsb::AdjointSession> adjoint_spare;  // device buffers of the last run, reused by the next
    cudaEvent_t fork = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_steps = -1, graph_collision_steps = -1;
    float graph_dt = -1.0f;
    uint32_t last_launches = 0;
    float last_kernel_ms = 0.0f;

    ~jsb_context();
};

namespace jsb {
namespace {

void free_groups(jsb_context *ctx) {
    for (auto &g : ctx->groups) {
        if (g.stream) cudaStreamDestroy(g.stream);
        if (g.done) cudaEventDestroy(g.done);
    }
    ctx->groups.clear();
}

void drop_graph(jsb_context *ctx) {
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
    ctx->graph_steps = -1;
}

size_t bucket_for(const jsb_context *ctx, uint32_t nv) {
    for (size_t i = 0; i < ctx->buckets.size(); ++i)
        if (nv <= ctx->buckets[i].max_vertices) return i;
    return ctx->buckets.size() - 1;
}

// The whole-step schedule body b walks, or null (pressure, a single iteration, the walk switched off,
// or a schedule level too wide for the 16-bit level descriptor).
const StepSchedRec *step_sched(const jsb_context *ctx, const BodyRec &b) {
    if (!ctx->step_walk || b.creation.pressure > 0.0f) return nullptr;
    const SettingsRec &s = *ctx->settings[b.settings_id];
    auto it = s.steps.find(b.creation.num_iterations);
    return it == s.steps.end() ? nullptr : it->second.get();
}

// Builds and uploads the whole-step schedules the bodies need (once per settings and iteration count).
jsb_status ensure_step_schedules(jsb_context *ctx) {
    if (!ctx->step_walk) return JSB_OK;
    for (const BodyRec &b : ctx->bodies) {
        if (b.creation.pressure > 0.0f || b.creation.num_iterations < 2) continue;
        SettingsRec &s = *ctx->settings[b.settings_id];
        if (s.steps.count(b.creation.num_iterations)) continue;
        auto rec = std::make_unique<StepSchedRec>();
        if (build_step_schedule(s.parsed, b.creation.num_iterations, rec->sched)) {
            JSB_CUDA(rec->levels.upload(reinterpret_cast<const uint4 *>(rec->sched.levels.data()), rec->sched.levels.size() / 4));
            JSB_CUDA(rec->records.upload(reinterpret_cast<const uint4 *>(rec->sched.records.data()), rec->sched.records.size() / 4));
            std::vector<uint32_t>().swap(rec->sched.records);  // the device copy is the one used
        } else {
            rec.reset();
        }
        s.steps[b.creation.num_iterations] = std::move(rec);
    }
    return JSB_OK;
}

inline float __uint_as_float_host(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

BodyDesc make_desc(const jsb_context *ctx, const BodyRec &b) {
    const SettingsRec &s = *ctx->settings[b.settings_id];
    BodyDesc d;
    d.levels = s.levels.ptr;  // padded device layout
    d.records = s.records.ptr;
    d.faces = s.faces.ptr;
    d.vf_off = s.vf_off_dev.ptr;
    d.vf = s.vf_dev.ptr;
    d.num_levels = s.schedule.num_levels;
    d.num_records = s.schedule.num_slots;
    const StepSchedRec *ss = step_sched(ctx, b);
    d.step_levels = ss ? ss->levels.ptr : nullptr;
    d.step_records = ss ? ss->records.ptr : nullptr;
    d.num_step_levels = ss ? ss->sched.num_levels : 0u;
    d.chunks = d.step_chunks = nullptr;  // set by attach_chunks for the ring of the body's launch group
    d.num_chunks = d.num_step_chunks = 0;
    d.stage_half = 0;
    d.num_faces = uint32_t(s.parsed.faces.size());
    d.num_vertices = uint32_t(s.parsed.vertices.size());
    d.vtx_offset = b.vtx_offset;
    d.num_iterations = b.creation.num_iterations;
    d.linear_damping = b.creation.linear_damping;
    d.max_linear_velocity = b.creation.max_linear_velocity;
    d.restitution = b.creation.restitution;
    d.friction = b.creation.friction;
    d.pressure = b.creation.pressure;
    d.gravity_factor = b.creation.gravity_factor;
    d.vertex_radius = b.creation.vertex_radius;
    d.flags = (b.creation.update_position ? kFlagUpdatePosition : 0u) | (b.creation.allow_sleeping ? kFlagAllowSleeping : 0u);
    const bool skinned = !s.parsed.skinned.empty() && ctx->skin_state.ptr;
    d.skin_params = skinned ? s.skin_params.ptr : nullptr;
    d.skin_state = skinned ? ctx->skin_state.ptr + size_t(b.vtx_offset) * 3 : nullptr;
    const size_t bi = size_t(&b - ctx->bodies.data());
    d.face_scratch = (b.creation.pressure > 0.0f && bi < ctx->face_off.size() && ctx->face_scratch.ptr)
                         ? ctx->face_scratch.ptr + ctx->face_off[bi]
                         : nullptr;
    return d;
}

constexpr size_t kStaticSmemReserve = 4096;  // static shared memory of the solver kernel

uint32_t pressure_faces(const SettingsRec &s, const BodyRec &b) {
    return b.creation.pressure > 0.0f ? uint32_t(s.parsed.faces.size()) : 0u;
}

constexpr uint32_t kMaxRingSlots = 256;
constexpr uint32_t kMaxCachedLevels = 4096;  // level descriptors a cluster CTA keeps in shared memory

constexpr uint32_t kMaxStepRingSlots = 512;  // whole-step levels are wider (slots beyond the ring are read in place)

uint32_t ring_slots_for(const SettingsRec &s) {
    uint32_t r = (s.schedule.max_level_slots + 31u) & ~31u;
    return std::max<uint32_t>(32u, std::min(r, kMaxRingSlots));
}

// Widest level of the schedule body b walks (rounded up to 32 slots, capped).
uint32_t ring_slots_for(const jsb_context *ctx, const BodyRec &b) {
    const SettingsRec &s = *ctx->settings[b.settings_id];
    const StepSchedRec *ss = step_sched(ctx, b);
    if (!ss) return ring_slots_for(s);
    uint32_t r = (ss->sched.max_level_slots + 31u) & ~31u;
    return std::max<uint32_t>(32u, std::min(r, kMaxStepRingSlots));
}

// Record slots per schedule-ring half wanted for body b: two of its widest levels, so that narrow levels
// stage several to a chunk.
uint32_t ring_half_for(const jsb_context *ctx, const BodyRec &b) { return 2 * ring_slots_for(ctx, b); }

constexpr uint32_t kMaxGrownRingSlots = 4096;  // 64 KB per half

// Record slots per half at which body b's chunks would average kStageLevels levels (its schedule's slots
// per level x kStageLevels, rounded up to 32, capped).
uint32_t ring_half_full(const jsb_context *ctx, const BodyRec &b) {
    const SettingsRec &s = *ctx->settings[b.settings_id];
    const StepSchedRec *ss = step_sched(ctx, b);
    const uint64_t slots = ss ? ss->sched.num_slots : s.schedule.num_slots;
    const uint64_t levels = std::max<uint64_t>(1, ss ? ss->sched.num_levels : s.schedule.num_levels);
    const uint64_t r = ((slots * kStageLevels / levels) + 31u) & ~uint64_t(31);
    return uint32_t(std::min<uint64_t>(r, kMaxGrownRingSlots));
}

// Staging chunks of a schedule for ring halves of `half` slots, built and uploaded once per half.
jsb_status chunk_table(std::map<uint32_t, std::pair<DevBuf<uint4>, uint32_t>> &cache, const std::vector<uint32_t> &levels,
                       uint32_t num_levels, bool per_substep, uint32_t half, const uint4 *&ptr, uint32_t &count) {
    auto it = cache.find(half);
    if (it == cache.end()) {
        std::vector<uint32_t> c = build_stage_chunks(levels, num_levels, per_substep, half);
        auto &e = cache[half];
        JSB_CUDA(e.first.upload(reinterpret_cast<const uint4 *>(c.data()), c.size() / 4));
        e.second = uint32_t(c.size() / 4);
        it = cache.find(half);
    }
    ptr = it->second.first.ptr;
    count = it->second.second;
    return JSB_OK;
}

// Points body bi's descriptor at the staging chunks of its schedules for ring halves of `half` slots.
jsb_status attach_chunks(jsb_context *ctx, uint32_t bi, uint32_t half) {
    BodyRec &b = ctx->bodies[bi];
    SettingsRec &s = *ctx->settings[b.settings_id];
    BodyDesc &d = ctx->descs_host[bi];
    d.stage_half = half;
    jsb_status st = chunk_table(s.chunks, s.schedule.padded_levels, s.schedule.num_levels, true, half, d.chunks, d.num_chunks);
    if (st != JSB_OK) return st;
    d.step_chunks = nullptr;
    d.num_step_chunks = 0;
    if (step_sched(ctx, b)) {
        StepSchedRec &ss = *s.steps[b.creation.num_iterations];
        st = chunk_table(ss.chunks, ss.sched.levels, ss.sched.num_levels, false, half, d.step_chunks, d.num_step_chunks);
    }
    return st;
}

double body_cost(const jsb_context *ctx, const BodyRec &b, int threads) {
    const SettingsRec &s = *ctx->settings[b.settings_id];
    double per_vertex = double(s.parsed.vertices.size()) / threads;
    double levels = 0;
    if (const StepSchedRec *ss = step_sched(ctx, b)) {
        const auto &lv = ss->sched.levels;
        for (uint32_t l = 0; l < ss->sched.num_levels; ++l) levels += double((lv[l * 4 + 3] + threads - 1) / threads);
        return levels + 6.0 * per_vertex;
    }
    const auto &lv = s.schedule.levels;
    for (uint32_t l = 0; l < s.schedule.num_levels; ++l) {
        uint32_t w = lv[(l + 1) * 4] - lv[l * 4];
        levels += double((w + threads - 1) / threads);
    }
    return double(b.creation.num_iterations) * (levels + 4.0 * per_vertex);
}

jsb_status rebuild_groups(jsb_context *ctx);

// Rebuilds the device-side body tables (and then the launch groups) after structural changes.
jsb_status rebuild(jsb_context *ctx) {
    if (!ctx->dirty) return ctx->groups_dirty ? rebuild_groups(ctx) : JSB_OK;
    drop_graph(ctx);
    free_groups(ctx);
    // vertex layout
    uint64_t total = 0;
    for (BodyRec &b : ctx->bodies) {
        b.vtx_offset = uint32_t(total);
        total += ctx->settings[b.settings_id]->parsed.vertices.size();
    }
    if (total > 0xffffffffull) return fail(JSB_ERR_CAPACITY, "more than 2^32 vertices in one context");
    // Keep existing device vertex state when only the tail grew (bodies are append-only).
    std::vector<float4> hx(total), hv(total);
    const uint64_t old_total = ctx->x.count;
    if (old_total) {
        JSB_CUDA(cudaMemcpy(hx.data(), ctx->x.ptr, old_total * sizeof(float4), cudaMemcpyDeviceToHost));
        JSB_CUDA(cudaMemcpy(hv.data(), ctx->v.ptr, old_total * sizeof(float4), cudaMemcpyDeviceToHost));
    }
    std::vector<BodyState> hstate(ctx->bodies.size());
    const size_t old_bodies = ctx->states.count;
    if (old_bodies)
        JSB_CUDA(cudaMemcpy(hstate.data(), ctx->states.ptr, old_bodies * sizeof(BodyState), cudaMemcpyDeviceToHost));
    for (size_t bi = 0; bi < ctx->bodies.size(); ++bi) {
        BodyRec &b = ctx->bodies[bi];
        const ParsedSettings &ps = ctx->settings[b.settings_id]->parsed;
        if (bi >= old_bodies) {
            hstate[bi] = b.state;
            for (size_t i = 0; i < ps.vertices.size(); ++i) {
                const auto &sv = ps.vertices[i];
                hx[b.vtx_offset + i] = make_float4(sv.pos[0], sv.pos[1], sv.pos[2], sv.inv_mass);
                hv[b.vtx_offset + i] = make_float4(sv.vel[0], sv.vel[1], sv.vel[2], 0.0f);
            }
        }
    }
    JSB_CUDA(ctx->x.upload(hx.data(), total));
    JSB_CUDA(ctx->v.upload(hv.data(), total));
    JSB_CUDA(ctx->prev.alloc(total));
    JSB_CUDA(ctx->plane.alloc(total));
    JSB_CUDA(ctx->shape.alloc(total));
    ctx->total_vertices = total;
    {  // skin states (SoftBodyMotionProperties::mSkinState, zero at creation) and switches; existing bodies keep theirs
        bool any = false;
        for (const BodyRec &b : ctx->bodies) any = any || !ctx->settings[b.settings_id]->parsed.skinned.empty();
        if (any) {
            std::vector<float4> hs(size_t(total) * 3, make_float4(0, 0, 0, 0));
            const size_t old = std::min(ctx->skin_state.count, hs.size());
            if (old) JSB_CUDA(cudaMemcpy(hs.data(), ctx->skin_state.ptr, old * sizeof(float4), cudaMemcpyDeviceToHost));
            JSB_CUDA(ctx->skin_state.upload(hs.data(), hs.size()));
        }
        std::vector<SkinCtl> hc(std::max<size_t>(ctx->bodies.size(), 1), SkinCtl{1.0f, kSkinEnabled});
        const size_t oldc = std::min(ctx->skin_ctl.count, hc.size());
        if (oldc) JSB_CUDA(cudaMemcpy(hc.data(), ctx->skin_ctl.ptr, oldc * sizeof(SkinCtl), cudaMemcpyDeviceToHost));
        JSB_CUDA(ctx->skin_ctl.upload(hc.data(), hc.size()));
    }
    {  // face scratch of the pressure bodies (used where a pressure body runs on the cluster path)
        size_t nf = 0;
        ctx->face_off.assign(ctx->bodies.size(), 0);
        for (size_t bi = 0; bi < ctx->bodies.size(); ++bi) {
            ctx->face_off[bi] = nf;
            if (ctx->bodies[bi].creation.pressure > 0.0f) nf += ctx->settings[ctx->bodies[bi].settings_id]->parsed.faces.size();
        }
        if (nf && ctx->face_scratch.count < nf) JSB_CUDA(ctx->face_scratch.alloc(nf));
    }
    jsb_status sst = ensure_step_schedules(ctx);
    if (sst != JSB_OK) return sst;
    ctx->descs_host.clear();
    for (const BodyRec &b : ctx->bodies) ctx->descs_host.push_back(make_desc(ctx, b));
    JSB_CUDA(ctx->descs.upload(ctx->descs_host.data(), ctx->descs_host.size()));
    JSB_CUDA(ctx->states.upload(hstate.data(), hstate.size()));
    {  // sleep records: existing bodies keep theirs, new bodies start awake with a zero timer
        std::vector<BodySleep> hs(ctx->bodies.size(), BodySleep{0.0f, 1u});
        const size_t old_sleep = std::min(ctx->sleep.count, hs.size());
        if (old_sleep) JSB_CUDA(cudaMemcpy(hs.data(), ctx->sleep.ptr, old_sleep * sizeof(BodySleep), cudaMemcpyDeviceToHost));
        JSB_CUDA(ctx->sleep.upload(hs.data(), hs.size()));
    }
    if (ctx->sensor_contact.count < std::max<size_t>(ctx->bodies.size(), 1)) {
        JSB_CUDA(ctx->sensor_contact.alloc(std::max<size_t>(ctx->bodies.size(), 1)));
        JSB_CUDA(cudaMemset(ctx->sensor_contact.ptr, 0, ctx->sensor_contact.count * sizeof(uint32_t)));
    }
    JSB_CUDA(ctx->colliders_dev.upload(ctx->colliders.data(), ctx->colliders.size()));
    ctx->pending_force.resize(ctx->bodies.size() * 3, 0.0f);
    if (ctx->pending_force_pinned) cudaFreeHost(ctx->pending_force_pinned);
    ctx->pending_force_pinned = nullptr;
    if (!ctx->bodies.empty()) JSB_CUDA(cudaMallocHost(&ctx->pending_force_pinned, ctx->bodies.size() * 3 * sizeof(float)));
    JSB_CUDA(ctx->forces.alloc(ctx->bodies.size() * 3));
    if (ctx->forces.count) JSB_CUDA(cudaMemset(ctx->forces.ptr, 0, ctx->forces.count * sizeof(float)));
    ctx->step_force_host.resize(ctx->bodies.size() * 3, 0.0f);
    JSB_CUDA(ctx->step_forces.upload(ctx->step_force_host.data(), ctx->step_force_host.size()));
    ctx->single_work_host.resize(ctx->bodies.size());
    for (size_t i = 0; i < ctx->bodies.size(); ++i) ctx->single_work_host[i] = uint32_t(i);
    JSB_CUDA(ctx->single_work.upload(ctx->single_work_host.data(), ctx->single_work_host.size()));
    if (!ctx->error.ptr) {
        JSB_CUDA(ctx->error.alloc(1));
        JSB_CUDA(cudaMemset(ctx->error.ptr, 0, sizeof(uint32_t)));
    }

    ctx->dirty = false;
    ctx->groups_dirty = true;
    return rebuild_groups(ctx);
}

// The launch group of the cluster path: one cluster per body; the cluster size is the configured one,
// or the largest (16, 8, 4, 2) that the device can co-schedule with the shared memory it needs.
jsb_status make_cluster_group(jsb_context *ctx, const std::vector<uint32_t> &bodies, size_t cap) {
    uint32_t max_nv = 0, max_levels = 0;
    for (uint32_t bi : bodies) {
        const SettingsRec &s = *ctx->settings[ctx->bodies[bi].settings_id];
        max_nv = std::max(max_nv, uint32_t(s.parsed.vertices.size()));
        max_levels = std::max(max_levels, s.schedule.num_levels);
    }
    const int T = ctx->cluster_threads;
    const int sizes[4] = {16, 8, 4, 2};
    for (int c : sizes) {
        if (ctx->cluster_size > 0 && c != ctx->cluster_size) continue;
        const uint32_t per_cta = std::max<uint32_t>(32u, (max_nv + uint32_t(c) - 1) / uint32_t(c));
        uint32_t shift = 5;
        while ((1u << shift) < per_cta) ++shift;
        uint32_t desc_cap = std::min<uint32_t>(max_levels + 2, kMaxCachedLevels);
        // Shrink the descriptor cache until the CTA fits.
        while (cluster_smem_bytes(shift, desc_cap) > cap && desc_cap > 0) desc_cap = desc_cap > 256 ? desc_cap - 256 : 0;
        const size_t smem = cluster_smem_bytes(shift, desc_cap);
        if (smem > cap || cluster_occupancy(c, T, smem) < 1) continue;
        ctx->groups.emplace_back();
        LaunchGroup &g = ctx->groups.back();
        g.cluster = c;
        g.threads = T;
        g.shift = shift;
        g.desc_cap = desc_cap;
        g.smem_vertices = max_nv;
        g.bodies = bodies;
        g.grid = c * int(bodies.size());
        JSB_CUDA(g.work.upload(g.bodies.data(), g.bodies.size()));
        JSB_CUDA(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
        return JSB_OK;
    }
    return fail(JSB_ERR_UNSUPPORTED, "a body with " + std::to_string(max_nv) + " vertices does not fit a thread-block cluster");
}

// One launch group per non-empty bucket: dynamic shared memory sized for its largest body, ring
// capacity for its widest level, bodies queued longest first.
jsb_status rebuild_groups(jsb_context *ctx) {
    drop_graph(ctx);
    free_groups(ctx);
    const size_t cap = ctx->max_smem_optin - kStaticSmemReserve;
    std::vector<std::vector<std::pair<double, uint32_t>>> members(ctx->buckets.size());
    std::vector<uint32_t> cluster_bodies;
    for (size_t bi = 0; bi < ctx->bodies.size(); ++bi) {
        const BodyRec &b = ctx->bodies[bi];
        const SettingsRec &s = *ctx->settings[b.settings_id];
        const uint32_t nv = uint32_t(s.parsed.vertices.size());
        size_t k = bucket_for(ctx, nv);
        // Bodies whose positions do not fit one CTA's shared memory take the cluster path.
        if (ctx->buckets[k].state_mode == 2 || step_smem_bytes(false, nv, pressure_faces(s, b), 32) > cap) {
            cluster_bodies.push_back(uint32_t(bi));
            continue;
        }
        members[k].push_back({body_cost(ctx, b, ctx->buckets[k].threads), uint32_t(bi)});
    }
    size_t one_cta_bodies = 0;
    for (auto &m : members) one_cta_bodies += m.size();
    for (size_t k = 0; k < ctx->buckets.size(); ++k) {
        if (members[k].empty()) continue;
        ctx->groups.emplace_back();
        LaunchGroup &g = ctx->groups.back();
        g.threads = ctx->buckets[k].threads;
        uint32_t widest = 32;
        for (auto &m : members[k]) {
            const BodyRec &b = ctx->bodies[m.second];
            const SettingsRec &s = *ctx->settings[b.settings_id];
            g.smem_vertices = std::max(g.smem_vertices, uint32_t(s.parsed.vertices.size()));
            g.smem_faces = std::max(g.smem_faces, pressure_faces(s, b));
            g.ring_slots = std::max(g.ring_slots, ring_half_for(ctx, b));
            widest = std::max(widest, ring_slots_for(ctx, b));
        }
        // Ring halves: two of the widest level wanted; shrink towards one widest level before giving up
        // shared-memory state, then further (wide levels are then staged in part and read in place).
        if (ctx->buckets[k].state_mode == 0)
            while (g.ring_slots > widest && step_smem_bytes(true, g.smem_vertices, g.smem_faces, g.ring_slots) > cap)
                g.ring_slots -= 32;
        while (g.ring_slots > 32 && step_smem_bytes(false, g.smem_vertices, g.smem_faces, g.ring_slots) > cap)
            g.ring_slots -= 32;
        g.smem_state = ctx->buckets[k].state_mode == 0 && step_smem_bytes(true, g.smem_vertices, g.smem_faces, g.ring_slots) <= cap;
        if (step_smem_bytes(g.smem_state, g.smem_vertices, g.smem_faces, g.ring_slots) > cap)
            return fail(JSB_ERR_UNSUPPORTED, "a body with " + std::to_string(g.smem_vertices) +
                                                 " vertices does not fit the shared-memory solver path");
        // Every chunk costs a wait and two bulk copies: when every body can have an SM to itself, grow
        // the halves towards chunks of kStageLevels levels while the CTA still fits an SM and the
        // placement of the state (in shared memory or not; also for the taped forward step, which
        // stages with the same ring) does not change; with at most one CTA per SM needed, CTAs per SM
        // do not matter. (In a batch of more bodies than SMs, larger rings cost co-resident CTAs of the
        // other buckets more than the fewer chunk turns save.)
        if (one_cta_bodies <= size_t(ctx->num_sms)) {
            uint32_t want = 0;
            for (auto &m : members[k]) want = std::max(want, ring_half_full(ctx, ctx->bodies[m.second]));
            const bool state_fits = step_smem_bytes(true, g.smem_vertices, g.smem_faces, g.ring_slots) <= cap;
            while (g.ring_slots < want) {
                const uint32_t r = std::min(want, g.ring_slots + std::max<uint32_t>(32, g.ring_slots / 2)) & ~31u;
                const size_t bytes = step_smem_bytes(g.smem_state, g.smem_vertices, g.smem_faces, r);
                if (r <= g.ring_slots || bytes > cap || step_occupancy(g.threads, g.smem_state, bytes) < 1 ||
                    (state_fits && step_smem_bytes(true, g.smem_vertices, g.smem_faces, r) > cap))
                    break;
                g.ring_slots = r;
            }
        }
        // Longest-processing-time-first order for the work queue.
        std::stable_sort(members[k].begin(), members[k].end(), [](const auto &a, const auto &b) { return a.first > b.first; });
        for (auto &m : members[k]) {
            g.bodies.push_back(m.second);
            jsb_status st = attach_chunks(ctx, m.second, g.ring_slots);
            if (st != JSB_OK) return st;
        }
        JSB_CUDA(g.work.upload(g.bodies.data(), g.bodies.size()));
        size_t smem = step_smem_bytes(g.smem_state, g.smem_vertices, g.smem_faces, g.ring_slots);
        int occ = step_occupancy(g.threads, g.smem_state, smem);
        if (occ <= 0) return fail(JSB_ERR_UNSUPPORTED, "solver kernel does not fit on an SM with this shared memory size");
        g.grid = int(std::min<size_t>(g.bodies.size(), size_t(occ) * ctx->num_sms));
        JSB_CUDA(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
    }
    if (!cluster_bodies.empty()) {
        jsb_status st = make_cluster_group(ctx, cluster_bodies, cap);
        if (st != JSB_OK) return st;
    }
    JSB_CUDA(ctx->descs.upload(ctx->descs_host.data(), ctx->descs_host.size()));
    // Larger buckets get higher stream priority (and are launched first): their bodies carry the
    // longest dependency chains, and a CTA sized for them needs an SM nobody else occupies.
    int least = 0, greatest = 0;
    JSB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int ng = int(ctx->groups.size());
    for (int gi = 0; gi < ng; ++gi) {
        int prio = least;
        if (ng > 1 && greatest != least) prio = least + (greatest - least) * gi / (ng - 1);
        JSB_CUDA(cudaStreamCreateWithPriority(&ctx->groups[gi].stream, cudaStreamNonBlocking, prio));
    }
    if (ctx->queues.count < std::max<size_t>(ctx->groups.size(), 1)) JSB_CUDA(ctx->queues.alloc(std::max<size_t>(ctx->groups.size(), 1)));
    ctx->groups_dirty = false;
    return JSB_OK;
}

StepParams base_params(jsb_context *ctx, float dt) {
    StepParams p;
    p.bodies = ctx->descs.ptr;
    p.states = ctx->states.ptr;
    p.x = ctx->x.ptr;
    p.v = ctx->v.ptr;
    p.prev = ctx->prev.ptr;
    p.plane = ctx->plane.ptr;
    p.shape = ctx->shape.ptr;
    p.colliders = ctx->colliders_dev.ptr;
    p.num_colliders = uint32_t(ctx->colliders.size());
    p.gravity[0] = ctx->gravity[0];
    p.gravity[1] = ctx->gravity[1];
    p.gravity[2] = ctx->gravity[2];
    p.dt = dt;
    p.error = ctx->error.ptr;
    p.forces = ctx->forces.ptr;
    p.step_forces = ctx->step_forces.ptr;
    p.ring_slots = kMaxRingSlots;
    p.tape = nullptr;
    p.tape_step = 0;
    p.sleep = ctx->sleep.ptr;
    p.sleep_velocity_threshold = ctx->sleep_velocity_threshold;
    p.time_before_sleep = ctx->time_before_sleep;
    const bool tables = !ctx->table_host.empty();
    p.tables = tables ? ctx->tables_dev.ptr : nullptr;
    p.table_slot = tables ? ctx->table_slot_dev.ptr : nullptr;
    p.dyn_list = tables ? ctx->dyn_list.ptr : nullptr;
    p.hulls = ctx->hulls_dev.ptr;
    p.hull_f4 = ctx->hull_f4_dev.ptr;
    p.hull_u32 = ctx->hull_u32_dev.ptr;
    const bool contacts = ctx->contact_readback && ctx->contact.count >= ctx->total_vertices;
    p.contact = contacts ? ctx->contact.ptr : nullptr;
    p.contact_point = contacts ? ctx->contact_point.ptr : nullptr;
    p.contact_delta = contacts ? ctx->contact_delta.ptr : nullptr;
    p.sensor_contact = tables ? ctx->sensor_contact.ptr : nullptr;
    p.skin_ctl = ctx->skin_ctl.ptr;
    return p;
}

// Buffers of the contact readback, sized for the current bodies (zeroed: no contact yet).
jsb_status ensure_contact_buffers(jsb_context *ctx) {
    if (!ctx->contact_readback) return JSB_OK;
    const size_t n = std::max<uint64_t>(ctx->total_vertices, 1), nb = std::max<size_t>(ctx->bodies.size(), 1);
    if (ctx->contact.count < n) {
        JSB_CUDA(ctx->contact.alloc(n));
        JSB_CUDA(cudaMemset(ctx->contact.ptr, 0, n));
        JSB_CUDA(ctx->contact_point.alloc(n));
    }
    if (ctx->contact_delta.count < 3 * nb) {
        JSB_CUDA(ctx->contact_delta.alloc(3 * nb));
        JSB_CUDA(cudaMemset(ctx->contact_delta.ptr, 0, 3 * nb * sizeof(float)));
    }
    return JSB_OK;
}

// Host-determined colliding shapes set since the last step: one ShapeTable per body that has them
// (slot order), uploaded on the step's stream ahead of its launches.
jsb_status upload_tables(jsb_context *ctx, cudaStream_t stream) {
    if (ctx->hulls_dirty) {  // registered hulls (synchronous: they are few and set up front)
        JSB_CUDA(ctx->hulls_dev.upload(ctx->hulls_host.data(), ctx->hulls_host.size()));
        JSB_CUDA(ctx->hull_f4_dev.upload(ctx->hull_f4_host.data(), ctx->hull_f4_host.size()));
        JSB_CUDA(ctx->hull_u32_dev.upload(ctx->hull_u32_host.data(), ctx->hull_u32_host.size()));
        ctx->hulls_dirty = false;
    }
    if (!ctx->tables_dirty) return JSB_OK;
    ctx->table_slot_host.assign(ctx->bodies.size(), -1);
    ctx->tables_staging.assign(ctx->table_host.size(), ShapeTable{});
    int32_t slot = 0;
    for (const auto &kv : ctx->table_host) {
        ShapeTable &t = ctx->tables_staging[size_t(slot)];
        t.count = uint32_t(kv.second.size());
        for (size_t k = 0; k < kv.second.size(); ++k) t.e[k] = kv.second[k];
        ctx->table_slot_host[kv.first] = slot++;
    }
    if (!ctx->tables_staging.empty()) {
        JSB_CUDA(ctx->tables_dev.ensure(ctx->tables_staging.size()));
        JSB_CUDA(cudaMemcpyAsync(ctx->tables_dev.ptr, ctx->tables_staging.data(), ctx->tables_staging.size() * sizeof(ShapeTable),
                                 cudaMemcpyHostToDevice, stream));
    }
    JSB_CUDA(ctx->table_slot_dev.ensure(std::max<size_t>(ctx->table_slot_host.size(), 1)));
    if (!ctx->table_slot_host.empty())
        JSB_CUDA(cudaMemcpyAsync(ctx->table_slot_dev.ptr, ctx->table_slot_host.data(), ctx->table_slot_host.size() * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, stream));
    JSB_CUDA(ctx->dyn_list.ensure(std::max<uint64_t>(ctx->total_vertices, 1)));
    ctx->tables_dirty = false;
    return JSB_OK;
}

// Enqueues one batched step (all launch groups) on `stream`.
jsb_status enqueue_batched(jsb_context *ctx, float dt, cudaStream_t stream, uint32_t &launches) {
    if (ctx->groups.empty()) return JSB_OK;
    JSB_CUDA(cudaMemsetAsync(ctx->queues.ptr, 0, ctx->queues.count * sizeof(uint32_t), stream));
    JSB_CUDA(cudaEventRecord(ctx->fork, stream));
    for (size_t k = ctx->groups.size(); k-- > 0;) {  // largest bucket first
        const size_t gi = k;
        LaunchGroup &g = ctx->groups[gi];
        JSB_CUDA(cudaStreamWaitEvent(g.stream, ctx->fork, 0));
        StepParams p = base_params(ctx, dt);
        p.work = g.work.ptr;
        p.num_work = uint32_t(g.bodies.size());
        p.queue = ctx->queues.ptr + gi;
        p.ring_slots = g.ring_slots;
        if (g.cluster > 0)
            JSB_CUDA(launch_cluster_step(p, g.cluster, g.threads, g.shift, g.desc_cap, g.stream));
        else
            JSB_CUDA(launch_step(p, g.threads, g.smem_state, g.smem_vertices, g.smem_faces, g.grid, g.stream));
        ++launches;
        JSB_CUDA(cudaEventRecord(g.done, g.stream));
        JSB_CUDA(cudaStreamWaitEvent(stream, g.done, 0));
    }
    return JSB_OK;
}

jsb_status upload_forces(jsb_context *ctx, cudaStream_t stream, bool &uploaded) {
    uploaded = false;
    if (!ctx->forces_pending) return JSB_OK;
    memcpy(ctx->pending_force_pinned, ctx->pending_force.data(), ctx->pending_force.size() * sizeof(float));
    JSB_CUDA(cudaMemcpyAsync(ctx->forces.ptr, ctx->pending_force_pinned, ctx->pending_force.size() * sizeof(float),
                             cudaMemcpyHostToDevice, stream));
    std::fill(ctx->pending_force.begin(), ctx->pending_force.end(), 0.0f);
    ctx->forces_pending = false;
    uploaded = true;
    return JSB_OK;
}

jsb_status step_impl(jsb_context *ctx, float dt, int collision_steps, cudaStream_t stream, bool plain, uint32_t &launches) {
    if (!(dt > 0.0f) || collision_steps < 1) return fail(JSB_ERR_INVALID_ARGUMENT, "dt must be > 0 and collision_steps >= 1");
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    if ((st = upload_tables(ctx, stream)) != JSB_OK) return st;
    if ((st = ensure_contact_buffers(ctx)) != JSB_OK) return st;
    const float step_dt = dt / float(collision_steps);
    for (int c = 0; c < collision_steps; ++c) {
        bool uploaded = false;
        if ((st = upload_forces(ctx, stream, uploaded)) != JSB_OK) return st;
        if (plain) {
            // One launch per body, one CTA each, on the caller's stream.
            for (size_t gi = 0; gi < ctx->groups.size(); ++gi) {
                LaunchGroup &g = ctx->groups[gi];
                for (uint32_t b : g.bodies) {
                    JSB_CUDA(cudaMemsetAsync(ctx->queues.ptr, 0, sizeof(uint32_t), stream));
                    StepParams p = base_params(ctx, step_dt);
                    p.work = ctx->single_work.ptr + b;
                    p.num_work = 1;
                    p.queue = ctx->queues.ptr;
                    const SettingsRec &s = *ctx->settings[ctx->bodies[b].settings_id];
                    p.ring_slots = g.ring_slots;  // the ring the body's staging chunks were built for
                    if (g.cluster > 0)
                        JSB_CUDA(launch_cluster_step(p, g.cluster, g.threads, g.shift, g.desc_cap, stream));
                    else
                        JSB_CUDA(launch_step(p, g.threads, g.smem_state, uint32_t(s.parsed.vertices.size()),
                                             pressure_faces(s, ctx->bodies[b]), 1, stream));
                    ++launches;
                }
            }
        } else if ((st = enqueue_batched(ctx, step_dt, stream, launches)) != JSB_OK)
            return st;
        if (uploaded) JSB_CUDA(cudaMemsetAsync(ctx->forces.ptr, 0, ctx->forces.count * sizeof(float), stream));
    }
    return JSB_OK;
}

// Enqueues one taped forward step of every body (tape position `tape_step` of the segment): one launch
// per group on the group's stream, forked from and joined back into `stream`.
jsb_status enqueue_taped(jsb_context *ctx, const AdjointSession &a, int tape_step, cudaStream_t stream, uint32_t &launches) {
    JSB_CUDA(cudaMemsetAsync(ctx->queues.ptr, 0, a.groups.size() * sizeof(uint32_t), stream));
    JSB_CUDA(cudaEventRecord(a.fork, stream));
    for (size_t gi = a.groups.size(); gi-- > 0;) {  // largest bodies first
        const AdjGroup &g = a.groups[gi];
        JSB_CUDA(cudaStreamWaitEvent(g.stream, a.fork, 0));
        StepParams p = base_params(ctx, a.dt);
        p.work = g.work.ptr;
        p.num_work = g.num_work;
        p.queue = ctx->queues.ptr + gi;
        p.ring_slots = g.ring_slots;
        p.tape = a.tape_desc.ptr;
        p.sleep = nullptr;  // (differentiable runs refuse bodies that may sleep)
        p.tape_step = uint32_t(tape_step);
        JSB_CUDA(launch_step_tape(p, g.threads, g.tape_smem_state, g.cap_vertices, g.cap_faces, g.tape_grid, g.stream));
        ++launches;
        JSB_CUDA(cudaEventRecord(g.done, g.stream));
        JSB_CUDA(cudaStreamWaitEvent(stream, g.done, 0));
    }
    return JSB_OK;
}

// Enqueues the adjoint of step `tape_step` of the segment for every body, like enqueue_taped.
jsb_status enqueue_adjoint(jsb_context *ctx, const AdjointSession &a, int tape_step, cudaStream_t stream, uint32_t &launches) {
    JSB_CUDA(cudaMemsetAsync(ctx->queues.ptr, 0, a.groups.size() * sizeof(uint32_t), stream));
    JSB_CUDA(cudaEventRecord(a.fork, stream));
    for (size_t gi = a.groups.size(); gi-- > 0;) {
        const AdjGroup &g = a.groups[gi];
        JSB_CUDA(cudaStreamWaitEvent(g.stream, a.fork, 0));
        AdjParams q;
        q.bodies = ctx->descs.ptr;
        q.tape = a.tape_desc.ptr;
        q.tape_step = uint32_t(tape_step);
        q.work = g.work.ptr;
        q.num_work = g.num_work;
        q.queue = ctx->queues.ptr + gi;
        q.adj_x = a.adj_x.ptr;
        q.adj_v = a.adj_v.ptr;
        q.grad_force = a.grad_force.ptr;
        for (int k = 0; k < 3; ++k) q.gravity[k] = ctx->gravity[k];
        q.dt = a.dt;
        q.ring_depth = g.adj_depth;
        q.ring_rpt = g.adj_rpt;
        JSB_CUDA(launch_adjoint(q, g.cap_vertices, g.cap_faces, g.adj_grid, g.threads, g.stream));
        ++launches;
        JSB_CUDA(cudaEventRecord(g.done, g.stream));
        JSB_CUDA(cudaStreamWaitEvent(stream, g.done, 0));
    }
    return JSB_OK;
}

jsb_context *check_ctx(jsb_context *ctx) {
    if (!ctx) g_last_error = "null context";
    return ctx;
}

}  // namespace
}  // namespace jsb

jsb_context::~jsb_context() {
    jsb::drop_graph(this);
    jsb::free_groups(this);
    if (fork) cudaEventDestroy(fork);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (pending_force_pinned) cudaFreeHost(pending_force_pinned);
}

using namespace jsb;

extern "C" {

const char *jsb_last_error_string(void) { return g_last_error.c_str(); }
const char *jsb_version(void) { return "jsb 0.1 (sm_103a)"; }

jsb_status jsb_context_create(int device, jsb_context **out) {
    if (!out) return fail(JSB_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(JSB_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= count) return fail(JSB_ERR_INVALID_ARGUMENT, "device index out of range");
    JSB_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    JSB_CUDA(cudaGetDeviceProperties(&prop, device));
    auto ctx = std::make_unique<jsb_context>();
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    ctx->max_smem_optin = prop.sharedMemPerBlockOptin;
    // Default launch shapes (the autotuner starts from this table and keeps only measured gains): wide
    // CTAs with only positions in shared memory for the larger bodies, whose whole-step levels hold up
    // to a few hundred slots; small CTAs for small bodies, many to an SM.
    ctx->buckets = {{128, 64, 1},   {256, 64, 1},   {512, 128, 1},  {1024, 256, 1}, {1536, 256, 1},
                    {2048, 256, 1}, {3072, 256, 1}, {4096, 256, 1}, {8192, 256, 1}, {65536, 256, 1}};
    // static shared memory of the solver kernel is under 4 KB
    JSB_CUDA(init_step_kernels(int(ctx->max_smem_optin - kStaticSmemReserve)));
    JSB_CUDA(init_adjoint_kernels(int(ctx->max_smem_optin - kStaticSmemReserve)));
    JSB_CUDA(init_cluster_kernels(int(ctx->max_smem_optin - kStaticSmemReserve)));
    JSB_CUDA(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
    JSB_CUDA(cudaEventCreate(&ctx->t0));
    JSB_CUDA(cudaEventCreate(&ctx->t1));
    *out = ctx.release();
    return JSB_OK;
}

jsb_status jsb_context_destroy(jsb_context *ctx) {
    if (!ctx) return fail(JSB_ERR_INVALID_ARGUMENT, "null context");
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    delete ctx;
    return JSB_OK;
}

jsb_status jsb_set_gravity(jsb_context *ctx, const float gravity[3]) {
    if (!check_ctx(ctx) || !gravity) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    memcpy(ctx->gravity, gravity, sizeof(ctx->gravity));
    drop_graph(ctx);
    return JSB_OK;
}

jsb_status jsb_settings_upload(jsb_context *ctx, const void *blob, size_t len, uint32_t *settings_id) {
    if (!check_ctx(ctx) || !settings_id) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    auto rec = std::make_unique<SettingsRec>();
    bool unsupported = false;
    std::string err = parse_settings(blob, len, rec->parsed, unsupported);
    if (!err.empty()) return fail(unsupported ? JSB_ERR_UNSUPPORTED : JSB_ERR_BLOB, err);
    rec->schedule = build_schedule(rec->parsed);
    const ParsedSettings &ps = rec->parsed;
    const size_t nv = ps.vertices.size();
    rec->vf_off.assign(nv + 1, 0);
    for (const auto &f : ps.faces)
        for (int k = 0; k < 3; ++k) rec->vf_off[f.v[k] + 1]++;
    for (size_t i = 0; i < nv; ++i) rec->vf_off[i + 1] += rec->vf_off[i];
    rec->vf.resize(rec->vf_off[nv]);
    std::vector<uint32_t> fill(rec->vf_off.begin(), rec->vf_off.end() - 1);
    for (size_t fi = 0; fi < ps.faces.size(); ++fi)
        for (int k = 0; k < 3; ++k) rec->vf[fill[ps.faces[fi].v[k]]++] = uint32_t(fi);
    std::vector<uint4> faces(ps.faces.size());
    for (size_t fi = 0; fi < ps.faces.size(); ++fi) faces[fi] = make_uint4(ps.faces[fi].v[0], ps.faces[fi].v[1], ps.faces[fi].v[2], 0);
    JSB_CUDA(cudaSetDevice(ctx->device));
    JSB_CUDA(rec->levels.upload(reinterpret_cast<const uint4 *>(rec->schedule.padded_levels.data()),
                                rec->schedule.padded_levels.size() / 4));
    JSB_CUDA(rec->records.upload(reinterpret_cast<const uint4 *>(rec->schedule.padded_records.data()),
                                 rec->schedule.padded_records.size() / 4));
    JSB_CUDA(rec->faces.upload(faces.data(), faces.size()));
    JSB_CUDA(rec->vf_off_dev.upload(rec->vf_off.data(), rec->vf_off.size()));
    JSB_CUDA(rec->vf_dev.upload(rec->vf.data(), rec->vf.size()));
    if (!ps.skinned.empty()) {
        std::vector<float4> sp(ps.skinned.size());
        for (size_t k = 0; k < sp.size(); ++k) {
            const auto &sk = ps.skinned[k];
            sp[k] = make_float4(sk.max_distance, sk.backstop_distance, sk.backstop_radius, __uint_as_float_host(sk.vertex));
        }
        JSB_CUDA(rec->skin_params.upload(sp.data(), sp.size()));
    }
    ctx->settings.push_back(std::move(rec));
    *settings_id = uint32_t(ctx->settings.size() - 1);
    return JSB_OK;
}

jsb_status jsb_body_add(jsb_context *ctx, uint32_t settings_id, const jsb_creation_settings *creation, const float position[3],
                        uint32_t *body_id) {
    if (!check_ctx(ctx) || !creation || !position || !body_id) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    if (settings_id >= ctx->settings.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "unknown settings id");
    if (creation->num_iterations < 1) return fail(JSB_ERR_INVALID_ARGUMENT, "num_iterations must be >= 1");
    if (!creation->make_rotation_identity)
        return fail(JSB_ERR_UNSUPPORTED, "bodies must keep an identity rotation (mMakeRotationIdentity = true)");
    BodyRec b;
    b.settings_id = settings_id;
    b.creation = *creation;
    memset(&b.state, 0, sizeof(b.state));
    for (int k = 0; k < 3; ++k) b.state.position[k] = position[k];
    // SoftBodyMotionProperties::Initialize: local bounds of the initial vertices, predicted = local.
    const ParsedSettings &ps = ctx->settings[settings_id]->parsed;
    for (int k = 0; k < 3; ++k) {
        b.state.bmin[k] = FLT_MAX;
        b.state.bmax[k] = -FLT_MAX;
    }
    for (const auto &v : ps.vertices)
        for (int k = 0; k < 3; ++k) {
            b.state.bmin[k] = b.state.bmin[k] < v.pos[k] ? b.state.bmin[k] : v.pos[k];
            b.state.bmax[k] = b.state.bmax[k] > v.pos[k] ? b.state.bmax[k] : v.pos[k];
        }
    for (int k = 0; k < 3; ++k) {
        b.state.pmin[k] = b.state.bmin[k];
        b.state.pmax[k] = b.state.bmax[k];
    }
    ctx->bodies.push_back(b);
    ctx->dirty = true;
    *body_id = uint32_t(ctx->bodies.size() - 1);
    return JSB_OK;
}

jsb_status jsb_collider_add(jsb_context *ctx, const jsb_collider *c, uint32_t *collider_id) {
    if (!check_ctx(ctx) || !c || !collider_id) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    if (c->type < JSB_COLLIDER_BOX || c->type > JSB_COLLIDER_CYLINDER) return fail(JSB_ERR_INVALID_ARGUMENT, "unknown collider type");
    ColliderDev d;
    d.type = c->type;
    for (int k = 0; k < 3; ++k) {
        d.position[k] = c->position[k];
        d.half_extent[k] = c->half_extent[k];
    }
    d.radius = c->radius;
    d.friction = c->friction;
    d.restitution = c->restitution;
    ctx->colliders.push_back(d);
    ctx->dirty = true;
    *collider_id = uint32_t(ctx->colliders.size() - 1);
    return JSB_OK;
}

jsb_status jsb_body_num_vertices(jsb_context *ctx, uint32_t body_id, uint32_t *n) {
    if (!check_ctx(ctx) || !n || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    *n = uint32_t(ctx->settings[ctx->bodies[body_id].settings_id]->parsed.vertices.size());
    return JSB_OK;
}

jsb_status jsb_body_add_force(jsb_context *ctx, uint32_t body_id, const float force[3]) {
    if (!check_ctx(ctx) || !force || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    for (int k = 0; k < 3; ++k) ctx->pending_force[body_id * 3 + k] += force[k];
    ctx->forces_pending = true;
    return JSB_OK;
}

jsb_status jsb_body_set_step_force(jsb_context *ctx, uint32_t body_id, const float force[3]) {
    if (!check_ctx(ctx) || !force || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    for (int k = 0; k < 3; ++k) ctx->step_force_host[body_id * 3 + k] = force[k];
    JSB_CUDA(cudaMemcpy(ctx->step_forces.ptr + body_id * 3, force, 3 * sizeof(float), cudaMemcpyHostToDevice));
    return JSB_OK;
}

jsb_status jsb_set_sleep_settings(jsb_context *ctx, float time_before_sleep, float point_velocity_sleep_threshold) {
    if (!check_ctx(ctx) || !(time_before_sleep >= 0.0f) || !(point_velocity_sleep_threshold >= 0.0f))
        return fail(JSB_ERR_INVALID_ARGUMENT, "sleep settings must be >= 0");
    drop_graph(ctx);  // graphs hold the launch parameters
    ctx->time_before_sleep = time_before_sleep;
    ctx->sleep_velocity_threshold = point_velocity_sleep_threshold;
    return JSB_OK;
}

jsb_status jsb_body_set_colliding_shapes(jsb_context *ctx, uint32_t body_id, const jsb_colliding_shape *shapes, uint32_t count) {
    static_assert(sizeof(jsb_colliding_shape) == sizeof(ShapeEntry), "jsb_colliding_shape and ShapeEntry share a layout");
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size() || (count && !shapes)) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    if (count > kMaxCollidingShapes) return fail(JSB_ERR_CAPACITY, "at most 16 colliding shapes per body");
    std::vector<ShapeEntry> t(count);
    for (uint32_t k = 0; k < count; ++k) {
        if (shapes[k].type < JSB_COLLIDER_BOX || shapes[k].type > JSB_COLLIDER_HULL)
            return fail(JSB_ERR_INVALID_ARGUMENT, "unknown collider type");
        if (shapes[k].type == JSB_COLLIDER_HULL && shapes[k].hull_id >= ctx->hulls_host.size())
            return fail(JSB_ERR_INVALID_ARGUMENT, "unknown hull id");
        if (shapes[k].motion_type < JSB_MOTION_STATIC || shapes[k].motion_type > JSB_MOTION_SENSOR)
            return fail(JSB_ERR_INVALID_ARGUMENT, "unknown motion type");
        std::memcpy(&t[k], &shapes[k], sizeof(ShapeEntry));
    }
    ctx->table_host[body_id] = std::move(t);
    ctx->tables_dirty = true;
    drop_graph(ctx);
    return JSB_OK;
}

jsb_status jsb_hull_add(jsb_context *ctx, const jsb_convex_hull *h, uint32_t *hull_id) {
    if (!check_ctx(ctx) || !h || !hull_id || !h->points || !h->planes || !h->face_vertex_counts || !h->face_vertices)
        return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    if (h->num_points < 4 || h->num_points > 256 || h->num_faces < 4 || h->num_faces > 255)
        return fail(JSB_ERR_INVALID_ARGUMENT, "a hull has 4 to 256 points and 4 to 255 faces");
    HullDev d;
    d.num_faces = h->num_faces;
    d.num_points = h->num_points;
    d.f4 = uint32_t(ctx->hull_f4_host.size());
    d.faces = uint32_t(ctx->hull_u32_host.size());
    std::vector<uint32_t> u32(2 * size_t(h->num_faces));
    uint32_t next = 0;
    for (uint32_t f = 0; f < h->num_faces; ++f) {
        const uint32_t n = h->face_vertex_counts[f];
        if (n < 3 || n > h->num_points) return fail(JSB_ERR_INVALID_ARGUMENT, "a hull face has 3 to num_points vertices");
        u32[2 * f] = d.faces + 2 * h->num_faces + next;
        u32[2 * f + 1] = n;
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t v = h->face_vertices[next + k];
            if (v >= h->num_points) return fail(JSB_ERR_INVALID_ARGUMENT, "hull face vertex out of range");
            u32.push_back(v);
        }
        next += n;
    }
    for (uint32_t f = 0; f < h->num_faces; ++f)
        ctx->hull_f4_host.push_back(make_float4(h->planes[4 * f], h->planes[4 * f + 1], h->planes[4 * f + 2], h->planes[4 * f + 3]));
    for (uint32_t i = 0; i < h->num_points; ++i)
        ctx->hull_f4_host.push_back(make_float4(h->points[3 * i], h->points[3 * i + 1], h->points[3 * i + 2], 0.0f));
    ctx->hull_u32_host.insert(ctx->hull_u32_host.end(), u32.begin(), u32.end());
    ctx->hulls_host.push_back(d);
    ctx->hulls_dirty = true;
    *hull_id = uint32_t(ctx->hulls_host.size() - 1);
    return JSB_OK;
}

// ---- skinning (SoftBodyMotionProperties::SkinVertices, :1139-1230) -------------------------------------
// Host arithmetic in the operation order of the reference's deterministic SSE build: Mat44 * Mat44 and
// Mat44 * Vec3 as ((c0 x + c1 y) + c2 z) + c3 (Mat44.inl:241-302), Vec3::Cross with separately rounded
// products, NormalizedOr with the length (x x + y y) + z z, a zero vector at or below FLT_MIN.
namespace {
struct V3h {
    float x, y, z;
};
inline V3h operator+(V3h a, V3h b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3h operator-(V3h a, V3h b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3h operator*(float s, V3h a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3h cross_h(V3h a, V3h b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3h normalized_or_zero(V3h v) {
    const float xx = v.x * v.x, yy = v.y * v.y, zz = v.z * v.z;
    const float len_sq = (xx + yy) + zz;
    if (len_sq <= FLT_MIN) return {0.0f, 0.0f, 0.0f};
    const float len = std::sqrt(len_sq);
    return {v.x / len, v.y / len, v.z / len};
}
struct M44h {
    float c[4][4];  // columns
};
inline M44h mat_mul_h(const M44h &a, const M44h &b) {
    M44h r;
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 4; ++k)
            r.c[i][k] = ((a.c[0][k] * b.c[i][0] + a.c[1][k] * b.c[i][1]) + a.c[2][k] * b.c[i][2]) + a.c[3][k] * b.c[i][3];
    return r;
}
inline V3h mat_vec_h(const M44h &a, V3h v) {
    float o[3];
    for (int k = 0; k < 3; ++k) o[k] = ((a.c[0][k] * v.x + a.c[1][k] * v.y) + a.c[2][k] * v.z) + a.c[3][k];
    return {o[0], o[1], o[2]};
}
}  // namespace

jsb_status jsb_body_skin_vertices(jsb_context *ctx, uint32_t body_id, const float *joint_matrices, uint32_t num_joints, int hard_skin_all) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size() || (num_joints && !joint_matrices))
        return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    const BodyRec &b = ctx->bodies[body_id];
    const ParsedSettings &ps = ctx->settings[b.settings_id]->parsed;
    if (ps.skinned.empty()) return fail(JSB_ERR_INVALID_ARGUMENT, "the body has no skinned constraints");
    std::vector<M44h> skin(ps.inv_binds.size());
    for (size_t k = 0; k < skin.size(); ++k) {
        const auto &ib = ps.inv_binds[k];
        if (ib.joint >= num_joints) return fail(JSB_ERR_INVALID_ARGUMENT, "inverse bind matrix refers to a joint out of range");
        M44h j, m;
        memcpy(j.c, joint_matrices + 16 * size_t(ib.joint), 64);
        memcpy(m.c, ib.m, 64);
        skin[k] = mat_mul_h(j, m);
    }
    const size_t nv = ps.vertices.size();
    JSB_CUDA(cudaDeviceSynchronize());
    std::vector<float4> hs(nv * 3);
    float4 *dev = ctx->skin_state.ptr + size_t(b.vtx_offset) * 3;
    JSB_CUDA(cudaMemcpy(hs.data(), dev, hs.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    auto get = [&](size_t i, int k) { return V3h{hs[i * 3 + k].x, hs[i * 3 + k].y, hs[i * 3 + k].z}; };
    auto put = [&](size_t i, int k, V3h v) { hs[i * 3 + k] = make_float4(v.x, v.y, v.z, 0.0f); };
    for (const auto &sk : ps.skinned) {
        const auto &bv = ps.vertices[sk.vertex];
        const V3h bind{bv.pos[0], bv.pos[1], bv.pos[2]};
        V3h pos{0.0f, 0.0f, 0.0f};
        for (const auto &w : sk.w) {
            if (w.weight == 0.0f) break;  // the first zero weight ends the list
            pos = pos + w.weight * mat_vec_h(skin[w.inv_bind], bind);
        }
        put(sk.vertex, 0, get(sk.vertex, 1));
        put(sk.vertex, 1, pos);
    }
    for (const auto &sk : ps.skinned) {
        V3h n{0.0f, 0.0f, 0.0f};
        const uint32_t nf = sk.normal_info >> 24;
        if (nf > 0) {
            for (uint32_t k = 0; k < nf; ++k) {
                const auto &f = ps.faces[ps.skinned_normals[(sk.normal_info & 0xffffffu) + k]];
                const V3h v0 = get(f.v[0], 1), v1 = get(f.v[1], 1), v2 = get(f.v[2], 1);
                n = n + normalized_or_zero(cross_h(v1 - v0, v2 - v0));
            }
            n = normalized_or_zero(n);
        }
        put(sk.vertex, 2, n);
    }
    SkinCtl ctl;
    JSB_CUDA(cudaMemcpy(&ctl, ctx->skin_ctl.ptr + body_id, sizeof(SkinCtl), cudaMemcpyDeviceToHost));
    const bool enabled = (ctl.flags & kSkinEnabled) != 0;
    if (hard_skin_all || !enabled) {  // hard skin every vertex (velocities reset), or only the kinematic ones
        std::vector<float4> hx(nv), hv(nv);
        JSB_CUDA(cudaMemcpy(hx.data(), ctx->x.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
        JSB_CUDA(cudaMemcpy(hv.data(), ctx->v.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
        for (const auto &sk : ps.skinned) {
            if (!hard_skin_all && sk.max_distance != 0.0f) continue;
            const V3h p = get(sk.vertex, 1);
            if (hard_skin_all) {
                put(sk.vertex, 0, p);
                hv[sk.vertex] = make_float4(0.0f, 0.0f, 0.0f, hv[sk.vertex].w);
            }
            hx[sk.vertex] = make_float4(p.x, p.y, p.z, hx[sk.vertex].w);
        }
        JSB_CUDA(cudaMemcpy(ctx->x.ptr + b.vtx_offset, hx.data(), nv * sizeof(float4), cudaMemcpyHostToDevice));
        JSB_CUDA(cudaMemcpy(ctx->v.ptr + b.vtx_offset, hv.data(), nv * sizeof(float4), cudaMemcpyHostToDevice));
    }
    JSB_CUDA(cudaMemcpy(dev, hs.data(), hs.size() * sizeof(float4), cudaMemcpyHostToDevice));
    ctl.flags |= kSkinPreviousValid;
    JSB_CUDA(cudaMemcpy(ctx->skin_ctl.ptr + body_id, &ctl, sizeof(SkinCtl), cudaMemcpyHostToDevice));
    drop_graph(ctx);
    return JSB_OK;
}

jsb_status jsb_body_set_skin_settings(jsb_context *ctx, uint32_t body_id, int enable_skin_constraints, float max_distance_multiplier) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    JSB_CUDA(cudaDeviceSynchronize());
    SkinCtl ctl;
    JSB_CUDA(cudaMemcpy(&ctl, ctx->skin_ctl.ptr + body_id, sizeof(SkinCtl), cudaMemcpyDeviceToHost));
    ctl.flags = (ctl.flags & ~kSkinEnabled) | (enable_skin_constraints ? kSkinEnabled : 0u);
    ctl.max_distance_multiplier = max_distance_multiplier;
    JSB_CUDA(cudaMemcpy(ctx->skin_ctl.ptr + body_id, &ctl, sizeof(SkinCtl), cudaMemcpyHostToDevice));
    drop_graph(ctx);
    return JSB_OK;
}

jsb_status jsb_body_sensor_contacts(jsb_context *ctx, uint32_t body_id, uint32_t *mask) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size() || !mask) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    *mask = 0;
    auto it = ctx->table_host.find(body_id);
    if (it == ctx->table_host.end() || ctx->dirty || ctx->sensor_contact.count <= body_id) return JSB_OK;
    JSB_CUDA(cudaSetDevice(ctx->device));
    JSB_CUDA(cudaDeviceSynchronize());
    JSB_CUDA(cudaMemcpy(mask, ctx->sensor_contact.ptr + body_id, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return JSB_OK;
}

jsb_status jsb_set_contact_readback(jsb_context *ctx, int enable) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    ctx->contact_readback = enable != 0;
    drop_graph(ctx);
    return JSB_OK;
}

jsb_status jsb_body_contacts(jsb_context *ctx, uint32_t body_id, uint8_t *has_contact, float *contact_points, float *normals,
                             int32_t *shape_index, float delta[3]) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    if (!ctx->contact_readback || ctx->contact.count < ctx->total_vertices || ctx->dirty)
        return fail(JSB_ERR_INVALID_ARGUMENT, "contact readback is off (jsb_set_contact_readback) or no step has run since");
    JSB_CUDA(cudaSetDevice(ctx->device));
    JSB_CUDA(cudaDeviceSynchronize());
    const BodyRec &b = ctx->bodies[body_id];
    const size_t nv = ctx->settings[b.settings_id]->parsed.vertices.size();
    std::vector<uint8_t> flag(nv);
    std::vector<float4> cp(nv), plane(nv);
    std::vector<int32_t> shape(nv);
    JSB_CUDA(cudaMemcpy(flag.data(), ctx->contact.ptr + b.vtx_offset, nv, cudaMemcpyDeviceToHost));
    JSB_CUDA(cudaMemcpy(cp.data(), ctx->contact_point.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
    JSB_CUDA(cudaMemcpy(plane.data(), ctx->plane.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
    JSB_CUDA(cudaMemcpy(shape.data(), ctx->shape.ptr + b.vtx_offset, nv * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (delta) JSB_CUDA(cudaMemcpy(delta, ctx->contact_delta.ptr + 3 * size_t(body_id), 3 * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < nv; ++i) {
        const bool c = flag[i] != 0;
        if (has_contact) has_contact[i] = c ? 1 : 0;
        for (int k = 0; k < 3; ++k) {
            const float pk = k == 0 ? cp[i].x : (k == 1 ? cp[i].y : cp[i].z);
            const float nk = k == 0 ? plane[i].x : (k == 1 ? plane[i].y : plane[i].z);
            if (contact_points) contact_points[3 * i + k] = c ? pk : 0.0f;
            if (normals) normals[3 * i + k] = c ? 0.0f - nk : 0.0f;  // GetContactNormal: -plane normal
        }
        if (shape_index) shape_index[i] = c ? shape[i] : -1;
    }
    return JSB_OK;
}

jsb_status jsb_body_clear_colliding_shapes(jsb_context *ctx, uint32_t body_id) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    if (ctx->table_host.erase(body_id)) ctx->tables_dirty = true;
    return JSB_OK;
}

jsb_status jsb_body_shape_velocities(jsb_context *ctx, uint32_t body_id, float *out, uint32_t *count) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size() || !out || !count) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    auto it = ctx->table_host.find(body_id);
    if (it == ctx->table_host.end() || ctx->tables_dirty || body_id >= ctx->table_slot_host.size() || ctx->table_slot_host[body_id] < 0)
        return fail(JSB_ERR_INVALID_ARGUMENT, "the body has not been stepped with host-determined colliding shapes");
    JSB_CUDA(cudaSetDevice(ctx->device));
    JSB_CUDA(cudaDeviceSynchronize());
    ShapeTable t;
    JSB_CUDA(cudaMemcpy(&t, ctx->tables_dev.ptr + ctx->table_slot_host[body_id], sizeof(ShapeTable), cudaMemcpyDeviceToHost));
    const bool dynamic = std::any_of(it->second.begin(), it->second.end(), [](const ShapeEntry &e) { return e.motion == kMotionDynamic; });
    *count = t.count;
    for (uint32_t k = 0; k < t.count; ++k) {
        const ShapeEntry &e = it->second[k];
        out[7 * k] = (t.updated >> k) & 1u ? 1.0f : 0.0f;
        for (int j = 0; j < 3; ++j) {  // (bodies without a dynamic shape leave the outputs untouched)
            out[7 * k + 1 + j] = dynamic ? t.lin[k][j] : e.lin[j];
            out[7 * k + 4 + j] = dynamic ? t.ang[k][j] : e.ang[j];
        }
    }
    return JSB_OK;
}

jsb_status jsb_body_is_active(jsb_context *ctx, uint32_t body_id, int *active) {
    if (!check_ctx(ctx) || !active || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    JSB_CUDA(cudaDeviceSynchronize());
    BodySleep sl;
    JSB_CUDA(cudaMemcpy(&sl, ctx->sleep.ptr + body_id, sizeof(BodySleep), cudaMemcpyDeviceToHost));
    *active = sl.active ? 1 : 0;
    return JSB_OK;
}

jsb_status jsb_body_set_active(jsb_context *ctx, uint32_t body_id, int active) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    JSB_CUDA(cudaDeviceSynchronize());
    BodySleep sl;
    JSB_CUDA(cudaMemcpy(&sl, ctx->sleep.ptr + body_id, sizeof(BodySleep), cudaMemcpyDeviceToHost));
    if (active) {
        sl = BodySleep{0.0f, 1u};  // ActivateBody resets the sleep timer (BodyManager.cpp:508-511)
    } else if (sl.active) {
        sl.active = 0u;  // DeactivateBody zeroes the body velocities (BodyManager.cpp:559-561)
        BodyState bs;
        JSB_CUDA(cudaMemcpy(&bs, ctx->states.ptr + body_id, sizeof(BodyState), cudaMemcpyDeviceToHost));
        memset(bs.lin_vel, 0, sizeof(bs.lin_vel));
        memset(bs.ang_vel, 0, sizeof(bs.ang_vel));
        JSB_CUDA(cudaMemcpy(ctx->states.ptr + body_id, &bs, sizeof(BodyState), cudaMemcpyHostToDevice));
    }
    JSB_CUDA(cudaMemcpy(ctx->sleep.ptr + body_id, &sl, sizeof(BodySleep), cudaMemcpyHostToDevice));
    return JSB_OK;
}

jsb_status jsb_step(jsb_context *ctx, float dt, int collision_steps, jsb_stream stream) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    JSB_CUDA(cudaSetDevice(ctx->device));
    uint32_t launches = 0;
    jsb_status st = step_impl(ctx, dt, collision_steps, reinterpret_cast<cudaStream_t>(stream), false, launches);
    ctx->last_launches = launches;
    return st;
}

jsb_status jsb_step_plain(jsb_context *ctx, float dt, int collision_steps, jsb_stream stream) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    JSB_CUDA(cudaSetDevice(ctx->device));
    uint32_t launches = 0;
    jsb_status st = step_impl(ctx, dt, collision_steps, reinterpret_cast<cudaStream_t>(stream), true, launches);
    ctx->last_launches = launches;
    return st;
}

jsb_status jsb_step_graph(jsb_context *ctx, float dt, int collision_steps, int num_steps, int repeats, jsb_stream stream_) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    if (num_steps < 1 || repeats < 0) return fail(JSB_ERR_INVALID_ARGUMENT, "num_steps must be >= 1, repeats >= 0");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    if (ctx->forces_pending)
        return fail(JSB_ERR_INVALID_ARGUMENT, "pending AddForce: forces are consumed per step; use jsb_step for forced steps");
    if (!ctx->table_host.empty())
        return fail(JSB_ERR_UNSUPPORTED, "host-determined colliding shapes change every step; use jsb_step");
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    uint32_t launches = 0;
    if (!ctx->graph_exec || ctx->graph_steps != num_steps || ctx->graph_dt != dt || ctx->graph_collision_steps != collision_steps) {
        drop_graph(ctx);
        cudaStream_t cap;
        JSB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cap);
            return fail(JSB_ERR_CUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
        }
        const float step_dt = dt / float(collision_steps);
        for (int s = 0; s < num_steps && st == JSB_OK; ++s)
            for (int c = 0; c < collision_steps && st == JSB_OK; ++c) st = enqueue_batched(ctx, step_dt, cap, launches);
        e = cudaStreamEndCapture(cap, &graph);
        cudaStreamDestroy(cap);
        if (st != JSB_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (e != cudaSuccess) return fail(JSB_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(JSB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        ctx->graph_steps = num_steps;
        ctx->graph_dt = dt;
        ctx->graph_collision_steps = collision_steps;
    } else {
        launches = uint32_t(ctx->groups.size()) * uint32_t(num_steps) * uint32_t(collision_steps);
    }
    JSB_CUDA(cudaEventRecord(ctx->t0, stream));
    for (int r = 0; r < repeats; ++r) JSB_CUDA(cudaGraphLaunch(ctx->graph_exec, stream));
    JSB_CUDA(cudaEventRecord(ctx->t1, stream));
    ctx->last_launches = launches * uint32_t(repeats);
    ctx->last_kernel_ms = -1.0f;
    if (repeats > 0) {
        JSB_CUDA(cudaEventSynchronize(ctx->t1));
        float ms = 0.0f;
        JSB_CUDA(cudaEventElapsedTime(&ms, ctx->t0, ctx->t1));
        ctx->last_kernel_ms = ms / float(repeats * num_steps);
    }
    return JSB_OK;
}

jsb_status jsb_synchronize(jsb_context *ctx) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    JSB_CUDA(cudaSetDevice(ctx->device));
    JSB_CUDA(cudaDeviceSynchronize());
    if (ctx->error.ptr) {
        uint32_t err = 0;
        JSB_CUDA(cudaMemcpy(&err, ctx->error.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        if (err) {
            JSB_CUDA(cudaMemset(ctx->error.ptr, 0, sizeof(uint32_t)));
            if (err & kErrTimeout) return fail(JSB_ERR_TIMEOUT, "a bounded device wait gave up");
            if (err & kErrNonFinite) return fail(JSB_ERR_NONFINITE, "non-finite vertex position or velocity");
            if (err & kErrShapeOverflow)
                return fail(JSB_ERR_CAPACITY, "more than " + std::to_string(kMaxCollidingShapes) + " colliding shapes for one body");
        }
    }
    return JSB_OK;
}

jsb_status jsb_body_bounds(jsb_context *ctx, uint32_t body_id, float local_bounds[6], float predicted_bounds[6]) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size() || !local_bounds || !predicted_bounds)
        return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    JSB_CUDA(cudaDeviceSynchronize());
    BodyState s;
    JSB_CUDA(cudaMemcpy(&s, ctx->states.ptr + body_id, sizeof(BodyState), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 3; ++k) {
        local_bounds[k] = s.bmin[k];
        local_bounds[3 + k] = s.bmax[k];
        predicted_bounds[k] = s.pmin[k];
        predicted_bounds[3 + k] = s.pmax[k];
    }
    return JSB_OK;
}

jsb_status jsb_body_read(jsb_context *ctx, uint32_t body_id, float position[3], float *local_positions, float *velocities) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    JSB_CUDA(cudaDeviceSynchronize());
    const BodyRec &b = ctx->bodies[body_id];
    const size_t nv = ctx->settings[b.settings_id]->parsed.vertices.size();
    if (position) {
        BodyState s;
        JSB_CUDA(cudaMemcpy(&s, ctx->states.ptr + body_id, sizeof(BodyState), cudaMemcpyDeviceToHost));
        memcpy(position, s.position, 3 * sizeof(float));
    }
    std::vector<float4> tmp(nv);
    if (local_positions) {
        JSB_CUDA(cudaMemcpy(tmp.data(), ctx->x.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nv; ++i) {
            local_positions[3 * i + 0] = tmp[i].x;
            local_positions[3 * i + 1] = tmp[i].y;
            local_positions[3 * i + 2] = tmp[i].z;
        }
    }
    if (velocities) {
        JSB_CUDA(cudaMemcpy(tmp.data(), ctx->v.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nv; ++i) {
            velocities[3 * i + 0] = tmp[i].x;
            velocities[3 * i + 1] = tmp[i].y;
            velocities[3 * i + 2] = tmp[i].z;
        }
    }
    return JSB_OK;
}

// SoftBodyMotionProperties::SaveState layout (single precision, no rods/skin):
//   MotionProperties::SaveState (Jolt/Physics/Body/MotionProperties.cpp:63-76): linear velocity (12),
//   angular velocity (12), force (12), torque (12), 3 sleep test spheres (48), sleep timer (4),
//   allow sleeping (1) = 101 bytes; then per vertex position (12) + velocity (12); then local bounds
//   and predicted bounds (4 x 12).
static constexpr size_t kMotionHeader = 101;

jsb_status jsb_body_save_state(jsb_context *ctx, uint32_t body_id, void *state, size_t capacity, size_t *len) {
    if (!check_ctx(ctx) || !len || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    const BodyRec &b = ctx->bodies[body_id];
    const size_t nv = ctx->settings[b.settings_id]->parsed.vertices.size();
    const bool skinned = !ctx->settings[b.settings_id]->parsed.skinned.empty();
    const size_t need = kMotionHeader + nv * 24 + (skinned ? nv * 36 : 0) + 48;
    *len = need;
    if (!state) return JSB_OK;
    if (capacity < need) return fail(JSB_ERR_INVALID_ARGUMENT, "state buffer too small");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    JSB_CUDA(cudaDeviceSynchronize());
    BodyState s;
    JSB_CUDA(cudaMemcpy(&s, ctx->states.ptr + body_id, sizeof(BodyState), cudaMemcpyDeviceToHost));
    std::vector<float4> hx(nv), hv(nv);
    JSB_CUDA(cudaMemcpy(hx.data(), ctx->x.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
    JSB_CUDA(cudaMemcpy(hv.data(), ctx->v.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
    uint8_t *o = static_cast<uint8_t *>(state);
    BodySleep sl;
    JSB_CUDA(cudaMemcpy(&sl, ctx->sleep.ptr + body_id, sizeof(BodySleep), cudaMemcpyDeviceToHost));
    memset(o, 0, kMotionHeader);
    memcpy(o + 0, s.lin_vel, 12);
    memcpy(o + 12, s.ang_vel, 12);
    memcpy(o + 96, &sl.timer, 4);  // mSleepTestTimer
    o[100] = b.creation.allow_sleeping;
    uint8_t *p = o + kMotionHeader;
    for (size_t i = 0; i < nv; ++i) {
        float pv[6] = {hx[i].x, hx[i].y, hx[i].z, hv[i].x, hv[i].y, hv[i].z};
        memcpy(p, pv, 24);
        p += 24;
    }
    if (skinned) {  // SkinState: previous position, position, normal (SoftBodyMotionProperties.cpp:1462-1467)
        std::vector<float4> hs(nv * 3);
        JSB_CUDA(cudaMemcpy(hs.data(), ctx->skin_state.ptr + size_t(b.vtx_offset) * 3, nv * 3 * sizeof(float4), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nv * 3; ++i) {
            memcpy(p, &hs[i], 12);
            p += 12;
        }
    }
    memcpy(p, s.bmin, 12);
    memcpy(p + 12, s.bmax, 12);
    memcpy(p + 24, s.pmin, 12);
    memcpy(p + 36, s.pmax, 12);
    return JSB_OK;
}

jsb_status jsb_body_restore_state(jsb_context *ctx, uint32_t body_id, const void *state, size_t len, const float position[3]) {
    if (!check_ctx(ctx) || !state || !position || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    const BodyRec &b = ctx->bodies[body_id];
    const ParsedSettings &ps = ctx->settings[b.settings_id]->parsed;
    const size_t nv = ps.vertices.size();
    const bool skinned = !ps.skinned.empty();
    if (len != kMotionHeader + nv * 24 + (skinned ? nv * 36 : 0) + 48)
        return fail(JSB_ERR_BLOB, "state size does not match the body's vertex count");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    JSB_CUDA(cudaDeviceSynchronize());
    const uint8_t *in = static_cast<const uint8_t *>(state);
    BodyState s;
    JSB_CUDA(cudaMemcpy(&s, ctx->states.ptr + body_id, sizeof(BodyState), cudaMemcpyDeviceToHost));
    memcpy(s.lin_vel, in + 0, 12);
    memcpy(s.ang_vel, in + 12, 12);
    memcpy(s.position, position, 12);
    BodySleep sl;  // the timer is restored; whether the body is active is the caller's (jsb_body_activate)
    JSB_CUDA(cudaMemcpy(&sl, ctx->sleep.ptr + body_id, sizeof(BodySleep), cudaMemcpyDeviceToHost));
    memcpy(&sl.timer, in + 96, 4);
    JSB_CUDA(cudaMemcpy(ctx->sleep.ptr + body_id, &sl, sizeof(BodySleep), cudaMemcpyHostToDevice));
    std::vector<float4> hx(nv), hv(nv);
    const uint8_t *p = in + kMotionHeader;
    for (size_t i = 0; i < nv; ++i) {
        float pv[6];
        memcpy(pv, p, 24);
        p += 24;
        hx[i] = make_float4(pv[0], pv[1], pv[2], ps.vertices[i].inv_mass);
        hv[i] = make_float4(pv[3], pv[4], pv[5], 0.0f);
    }
    if (skinned) {
        std::vector<float4> hs(nv * 3, make_float4(0, 0, 0, 0));
        for (size_t i = 0; i < nv * 3; ++i) {
            memcpy(&hs[i], p, 12);
            p += 12;
        }
        JSB_CUDA(cudaMemcpy(ctx->skin_state.ptr + size_t(b.vtx_offset) * 3, hs.data(), nv * 3 * sizeof(float4), cudaMemcpyHostToDevice));
    }
    memcpy(s.bmin, p, 12);
    memcpy(s.bmax, p + 12, 12);
    memcpy(s.pmin, p + 24, 12);
    memcpy(s.pmax, p + 36, 12);
    JSB_CUDA(cudaMemcpy(ctx->x.ptr + b.vtx_offset, hx.data(), nv * sizeof(float4), cudaMemcpyHostToDevice));
    JSB_CUDA(cudaMemcpy(ctx->v.ptr + b.vtx_offset, hv.data(), nv * sizeof(float4), cudaMemcpyHostToDevice));
    JSB_CUDA(cudaMemcpy(ctx->states.ptr + body_id, &s, sizeof(BodyState), cudaMemcpyHostToDevice));
    return JSB_OK;
}

jsb_status jsb_total_vertices(jsb_context *ctx, uint64_t *total) {
    if (!check_ctx(ctx) || !total) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    uint64_t t = 0;
    for (const BodyRec &b : ctx->bodies) t += ctx->settings[b.settings_id]->parsed.vertices.size();
    *total = t;
    return JSB_OK;
}

jsb_status jsb_state_upload_all(jsb_context *ctx, const float *local_positions, const float *velocities, jsb_stream stream_) {
    if (!check_ctx(ctx) || !local_positions || !velocities) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    const uint64_t n = ctx->total_vertices;
    if (ctx->staging3.count < 6 * n) JSB_CUDA(ctx->staging3.alloc(6 * n));
    JSB_CUDA(cudaMemcpyAsync(ctx->staging3.ptr, local_positions, 3 * n * sizeof(float), cudaMemcpyHostToDevice, stream));
    JSB_CUDA(cudaMemcpyAsync(ctx->staging3.ptr + 3 * n, velocities, 3 * n * sizeof(float), cudaMemcpyHostToDevice, stream));
    JSB_CUDA(launch_unpack_state(ctx->staging3.ptr, ctx->staging3.ptr + 3 * n, ctx->x.ptr, ctx->v.ptr, n, ctx->num_sms, stream));
    return JSB_OK;
}

jsb_status jsb_state_download_all(jsb_context *ctx, float *local_positions, float *velocities, jsb_stream stream_) {
    if (!check_ctx(ctx) || !local_positions || !velocities) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    const uint64_t n = ctx->total_vertices;
    if (ctx->staging3.count < 6 * n) JSB_CUDA(ctx->staging3.alloc(6 * n));
    JSB_CUDA(launch_pack_state(ctx->x.ptr, ctx->v.ptr, ctx->staging3.ptr, ctx->staging3.ptr + 3 * n, n, ctx->num_sms, stream));
    JSB_CUDA(cudaMemcpyAsync(local_positions, ctx->staging3.ptr, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, stream));
    JSB_CUDA(cudaMemcpyAsync(velocities, ctx->staging3.ptr + 3 * n, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, stream));
    return JSB_OK;
}

jsb_status jsb_body_positions_all(jsb_context *ctx, float *positions) {
    if (!check_ctx(ctx) || !positions) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    std::vector<BodyState> hs(ctx->bodies.size());
    if (!hs.empty()) JSB_CUDA(cudaMemcpy(hs.data(), ctx->states.ptr, hs.size() * sizeof(BodyState), cudaMemcpyDeviceToHost));
    for (size_t b = 0; b < hs.size(); ++b)
        for (int k = 0; k < 3; ++k) positions[3 * b + k] = hs[b].position[k];
    return JSB_OK;
}

jsb_status jsb_body_schedule_info(jsb_context *ctx, uint32_t body_id, uint32_t *num_levels, uint32_t *num_constraints) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    const Schedule &s = ctx->settings[ctx->bodies[body_id].settings_id]->schedule;
    if (num_levels) *num_levels = s.num_levels;
    if (num_constraints) *num_constraints = s.num_records;
    return JSB_OK;
}

jsb_status jsb_settings_schedule(const void *blob, size_t len, uint32_t *num_levels, uint32_t *num_records, uint32_t *levels,
                                 uint32_t *records, uint32_t *source) {
    if (!num_levels || !num_records) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    ParsedSettings ps;
    bool unsupported = false;
    std::string err = parse_settings(blob, len, ps, unsupported);
    if (!err.empty()) return fail(unsupported ? JSB_ERR_UNSUPPORTED : JSB_ERR_BLOB, err);
    Schedule s = build_schedule(ps);
    *num_levels = s.num_levels;
    *num_records = s.num_records;
    if (levels) memcpy(levels, s.levels.data(), s.levels.size() * sizeof(uint32_t));
    if (records) memcpy(records, s.records.data(), s.records.size() * sizeof(uint32_t));
    if (source) memcpy(source, s.source.data(), s.source.size() * sizeof(uint32_t));
    return JSB_OK;
}

jsb_status jsb_settings_regroup(const void *blob, size_t len, void *out, size_t capacity, size_t *out_len, uint32_t *remap) {
    if (!out_len) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    ParsedSettings ps;
    bool unsupported = false;
    std::string err = parse_settings(blob, len, ps, unsupported);
    if (!err.empty()) return fail(unsupported ? JSB_ERR_UNSUPPORTED : JSB_ERR_BLOB, err);
    if (!ps.skinned.empty()) return fail(JSB_ERR_UNSUPPORTED, "settings with skinned constraints are not regrouped");
    std::vector<uint32_t> map;
    const std::vector<uint8_t> bytes = regroup_settings(ps, map);
    *out_len = bytes.size();
    if (!out) return JSB_OK;
    if (capacity < bytes.size()) return fail(JSB_ERR_CAPACITY, "output buffer too small");
    memcpy(out, bytes.data(), bytes.size());
    if (remap) memcpy(remap, map.data(), map.size() * sizeof(uint32_t));
    return JSB_OK;
}

jsb_status jsb_settings_step_schedule(const void *blob, size_t len, uint32_t num_iterations, uint32_t *num_levels,
                                      uint32_t *num_slots, uint32_t *levels, uint32_t *records, uint32_t *source) {
    if (!num_levels || !num_slots) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    ParsedSettings ps;
    bool unsupported = false;
    std::string err = parse_settings(blob, len, ps, unsupported);
    if (!err.empty()) return fail(unsupported ? JSB_ERR_UNSUPPORTED : JSB_ERR_BLOB, err);
    StepSchedule s;
    if (!build_step_schedule(ps, num_iterations, s, source != nullptr)) {
        *num_levels = 0;
        *num_slots = 0;
        return JSB_OK;
    }
    *num_levels = s.num_levels;
    *num_slots = s.num_slots;
    if (levels) memcpy(levels, s.levels.data(), s.levels.size() * sizeof(uint32_t));
    if (records) memcpy(records, s.records.data(), s.records.size() * sizeof(uint32_t));
    if (source) memcpy(source, s.source.data(), s.source.size() * sizeof(uint32_t));
    return JSB_OK;
}

jsb_status jsb_set_bucket_config(jsb_context *ctx, uint32_t max_vertices, uint32_t threads, uint32_t state_mode) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    if (threads != 32 && threads != 64 && threads != 128 && threads != 256 && threads != 512)
        return fail(JSB_ERR_INVALID_ARGUMENT, "threads must be 32, 64, 128, 256 or 512");
    if (state_mode > 2) return fail(JSB_ERR_INVALID_ARGUMENT, "state_mode must be 0, 1 or 2");
    bool found = false;
    for (Bucket &b : ctx->buckets)
        if (b.max_vertices == max_vertices) {
            b.threads = int(threads);
            b.state_mode = int(state_mode);
            found = true;
        }
    if (!found) ctx->buckets.push_back({max_vertices, int(threads), int(state_mode)});
    std::sort(ctx->buckets.begin(), ctx->buckets.end(), [](const Bucket &a, const Bucket &b) { return a.max_vertices < b.max_vertices; });
    ctx->groups_dirty = true;
    return JSB_OK;
}

jsb_status jsb_set_cluster_config(jsb_context *ctx, uint32_t cluster_size, uint32_t threads) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    if (cluster_size != 0 && cluster_size != 2 && cluster_size != 4 && cluster_size != 8 && cluster_size != 16)
        return fail(JSB_ERR_INVALID_ARGUMENT, "cluster_size must be 0 (automatic), 2, 4, 8 or 16");
    if (threads != 128 && threads != 256 && threads != 512)
        return fail(JSB_ERR_INVALID_ARGUMENT, "threads must be 128, 256 or 512 on the cluster path");
    ctx->cluster_size = int(cluster_size);
    ctx->cluster_threads = int(threads);
    ctx->groups_dirty = true;
    return JSB_OK;
}

jsb_status jsb_set_step_walk(jsb_context *ctx, int enable) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    if (ctx->step_walk == (enable != 0)) return JSB_OK;
    if (ctx->adjoint) return fail(JSB_ERR_INVALID_ARGUMENT, "the walk cannot change during a differentiable run (jsb_adjoint_end first)");
    ctx->step_walk = enable != 0;
    ctx->dirty = true;  // body descriptors and launch groups change
    return JSB_OK;
}

jsb_status jsb_get_cluster_config(jsb_context *ctx, uint32_t *cluster_size, uint32_t *threads, uint32_t *num_bodies) {
    if (!check_ctx(ctx) || !cluster_size || !threads || !num_bodies) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    *cluster_size = uint32_t(ctx->cluster_size);
    *threads = uint32_t(ctx->cluster_threads);
    *num_bodies = 0;
    for (const LaunchGroup &g : ctx->groups)
        if (g.cluster > 0) {
            *cluster_size = uint32_t(g.cluster);
            *threads = uint32_t(g.threads);
            *num_bodies = uint32_t(g.bodies.size());
        }
    return JSB_OK;
}

jsb_status jsb_set_bucket_threads(jsb_context *ctx, uint32_t max_vertices, uint32_t threads) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    uint32_t mode = 0;
    for (const Bucket &b : ctx->buckets)
        if (b.max_vertices == max_vertices) mode = uint32_t(b.state_mode);
    return jsb_set_bucket_config(ctx, max_vertices, threads, mode);
}

jsb_status jsb_get_bucket_config(jsb_context *ctx, uint32_t index, uint32_t *max_vertices, uint32_t *threads, uint32_t *state_mode) {
    if (!check_ctx(ctx) || !max_vertices || !threads || !state_mode) return fail(JSB_ERR_INVALID_ARGUMENT, "null argument");
    if (index >= ctx->buckets.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bucket index out of range");
    *max_vertices = ctx->buckets[index].max_vertices;
    *threads = uint32_t(ctx->buckets[index].threads);
    *state_mode = uint32_t(ctx->buckets[index].state_mode);
    return JSB_OK;
}

jsb_status jsb_last_launch_count(jsb_context *ctx, uint32_t *launches) {
    if (!check_ctx(ctx) || !launches) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    *launches = ctx->last_launches;
    return JSB_OK;
}

jsb_status jsb_last_kernel_ms(jsb_context *ctx, float *ms) {
    if (!check_ctx(ctx) || !ms) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    *ms = ctx->last_kernel_ms;
    return JSB_OK;
}

// Autotuner: coordinate descent over the bucket table. For every occupied bucket (largest first) each
// launch shape -- threads per CTA in {32, 64, 128, 256, 512} x vertex state in shared / global memory -- is
// tried with the other buckets fixed, and the one giving the fastest whole batched step (all buckets
// running concurrently, as in jsb_step) is kept. Device state is saved before and restored after.
jsb_status jsb_autotune(jsb_context *ctx, float dt, int trials) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    if (trials < 1) trials = 1;
    if (!(dt > 0.0f)) return fail(JSB_ERR_INVALID_ARGUMENT, "dt must be > 0");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    if (ctx->bodies.empty()) return JSB_OK;
    const uint64_t n = ctx->total_vertices;
    DevBuf<float4> sx, sv;
    DevBuf<BodyState> ss;
    JSB_CUDA(sx.alloc(n));
    JSB_CUDA(sv.alloc(n));
    JSB_CUDA(ss.alloc(ctx->bodies.size()));
    JSB_CUDA(cudaMemcpy(sx.ptr, ctx->x.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemcpy(sv.ptr, ctx->v.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemcpy(ss.ptr, ctx->states.ptr, ctx->bodies.size() * sizeof(BodyState), cudaMemcpyDeviceToDevice));
    cudaStream_t stream;
    JSB_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    // Every configuration is timed on the same steps: the saved state is restored before each one.
    auto measure = [&](float &ms_out) -> jsb_status {
        jsb_status s2 = rebuild_groups(ctx);
        if (s2 != JSB_OK) return s2;
        JSB_CUDA(cudaMemcpyAsync(ctx->x.ptr, sx.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream));
        JSB_CUDA(cudaMemcpyAsync(ctx->v.ptr, sv.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice, stream));
        JSB_CUDA(cudaMemcpyAsync(ctx->states.ptr, ss.ptr, ctx->bodies.size() * sizeof(BodyState), cudaMemcpyDeviceToDevice,
                                 stream));
        std::vector<float> times;
        for (int k = 0; k < trials + 1; ++k) {
            uint32_t launches = 0;
            JSB_CUDA(cudaEventRecord(ctx->t0, stream));
            if ((s2 = enqueue_batched(ctx, dt, stream, launches)) != JSB_OK) return s2;
            JSB_CUDA(cudaEventRecord(ctx->t1, stream));
            JSB_CUDA(cudaEventSynchronize(ctx->t1));
            float ms = 0.0f;
            JSB_CUDA(cudaEventElapsedTime(&ms, ctx->t0, ctx->t1));
            if (k > 0) times.push_back(ms);  // the first launch is a warm-up
        }
        std::sort(times.begin(), times.end());
        ms_out = times[times.size() / 2];
        return JSB_OK;
    };
    std::vector<size_t> occupied;
    for (size_t k = 0; k < ctx->buckets.size(); ++k)
        for (const BodyRec &b : ctx->bodies)
            if (bucket_for(ctx, uint32_t(ctx->settings[b.settings_id]->parsed.vertices.size())) == k) {
                occupied.push_back(k);
                break;
            }
    float best_ms = 0.0f;
    st = measure(best_ms);
    // Starting points: the current table and a few uniform ones (buckets interact through SM sharing,
    // so coordinate descent from a single start can stall in a poor local optimum).
    {
        const std::vector<Bucket> current = ctx->buckets;
        std::vector<Bucket> best_table = current;
        for (int variant = 0; variant < 5 && st == JSB_OK; ++variant) {
            std::vector<Bucket> t = current;
            for (Bucket &b : t) {
                if (b.state_mode == 2) continue;
                const bool large = b.max_vertices >= 1024;
                switch (variant) {
                    case 0: b.state_mode = 1; break;  // positions only in shared memory: more CTAs per SM
                    case 1: b.state_mode = 1, b.threads = large ? 128 : 32; break;
                    case 2: b.state_mode = 1, b.threads = large ? 256 : 64; break;
                    case 3: b.state_mode = 1, b.threads = large ? 512 : 64; break;
                    default: b.state_mode = 0, b.threads = large ? 128 : 32; break;
                }
            }
            ctx->buckets = t;
            float ms = 0.0f;
            st = measure(ms);
            if (st == JSB_OK && ms < best_ms) {
                best_ms = ms;
                best_table = t;
            }
        }
        ctx->buckets = best_table;
    }
    // Coordinate descent over each occupied bucket's (threads, state placement), largest bucket first,
    // for up to two rounds.
    const int choices[5] = {32, 64, 128, 256, 512};
    for (int round = 0; round < 2 && st == JSB_OK; ++round) {
        bool improved = false;
        for (auto it = occupied.rbegin(); st == JSB_OK && it != occupied.rend(); ++it) {
            Bucket &bk = ctx->buckets[*it];
            if (bk.state_mode == 2) continue;
            Bucket best = bk;
            for (int mode = 0; mode < 2 && st == JSB_OK; ++mode)
                for (int t : choices) {
                    if (t == best.threads && mode == best.state_mode) continue;
                    bk.threads = t;
                    bk.state_mode = mode;
                    float ms = 0.0f;
                    st = measure(ms);
                    if (st != JSB_OK) break;
                    if (ms < best_ms) {
                        best_ms = ms;
                        best = bk;
                        improved = true;
                    }
                }
            bk = best;
        }
        if (!improved) break;
    }
    cudaStreamDestroy(stream);
    JSB_CUDA(cudaMemcpy(ctx->x.ptr, sx.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemcpy(ctx->v.ptr, sv.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemcpy(ctx->states.ptr, ss.ptr, ctx->bodies.size() * sizeof(BodyState), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemset(ctx->error.ptr, 0, sizeof(uint32_t)));
    if (st != JSB_OK) return st;
    ctx->groups_dirty = true;
    return rebuild(ctx);
}

// ---- differentiable runs ----------------------------------------------------------------------------

jsb_status jsb_body_set_compliance(jsb_context *ctx, uint32_t body_id, const float *edge_compliance, uint32_t num_edges,
                                   const float *volume_compliance, uint32_t num_volumes) {
    if (!check_ctx(ctx) || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    const uint32_t sid = ctx->bodies[body_id].settings_id;
    for (size_t b = 0; b < ctx->bodies.size(); ++b)
        if (b != body_id && ctx->bodies[b].settings_id == sid)
            return fail(JSB_ERR_INVALID_ARGUMENT, "settings are shared with another body; upload a separate copy to change compliance");
    SettingsRec &s = *ctx->settings[sid];
    if ((edge_compliance && num_edges != s.parsed.edges.size()) || (volume_compliance && num_volumes != s.parsed.volumes.size()))
        return fail(JSB_ERR_INVALID_ARGUMENT, "compliance arrays must cover every edge / volume constraint");
    JSB_CUDA(cudaSetDevice(ctx->device));
    JSB_CUDA(cudaDeviceSynchronize());
    if (edge_compliance)
        for (uint32_t i = 0; i < num_edges; ++i) s.parsed.edges[i].compliance = edge_compliance[i];
    if (volume_compliance)
        for (uint32_t i = 0; i < num_volumes; ++i) s.parsed.volumes[i].compliance = volume_compliance[i];
    s.schedule = build_schedule(s.parsed);  // same layout, new compliance words
    JSB_CUDA(cudaMemcpy(s.records.ptr, s.schedule.padded_records.data(), s.schedule.padded_records.size() * sizeof(uint32_t),
                        cudaMemcpyHostToDevice));
    for (auto &kv : s.steps) {
        if (!kv.second) continue;
        StepSchedRec &r = *kv.second;
        if (!build_step_schedule(s.parsed, kv.first, r.sched)) return fail(JSB_ERR_CAPACITY, "whole-step schedule rebuild failed");
        JSB_CUDA(cudaMemcpy(r.records.ptr, r.sched.records.data(), r.sched.records.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        std::vector<uint32_t>().swap(r.sched.records);
    }
    drop_graph(ctx);
    return JSB_OK;
}

namespace {

jsb_status save_state(jsb_context *ctx, DevBuf<float4> &x, DevBuf<float4> &v, DevBuf<BodyState> &st) {
    const uint64_t n = ctx->total_vertices;
    JSB_CUDA(x.ensure(n));
    JSB_CUDA(v.ensure(n));
    JSB_CUDA(st.ensure(ctx->bodies.size()));
    JSB_CUDA(cudaMemcpy(x.ptr, ctx->x.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemcpy(v.ptr, ctx->v.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemcpy(st.ptr, ctx->states.ptr, ctx->bodies.size() * sizeof(BodyState), cudaMemcpyDeviceToDevice));
    return JSB_OK;
}

jsb_status load_state(jsb_context *ctx, const DevBuf<float4> &x, const DevBuf<float4> &v, const DevBuf<BodyState> &st) {
    const uint64_t n = ctx->total_vertices;
    JSB_CUDA(cudaMemcpy(ctx->x.ptr, x.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemcpy(ctx->v.ptr, v.ptr, n * sizeof(float4), cudaMemcpyDeviceToDevice));
    JSB_CUDA(cudaMemcpy(ctx->states.ptr, st.ptr, ctx->bodies.size() * sizeof(BodyState), cudaMemcpyDeviceToDevice));
    return JSB_OK;
}

}  // namespace

jsb_status jsb_adjoint_begin(jsb_context *ctx, float dt, int num_steps, int checkpoint_every) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    if (!(dt > 0.0f) || num_steps < 1 || checkpoint_every < 1)
        return fail(JSB_ERR_INVALID_ARGUMENT, "dt must be > 0, num_steps >= 1 and checkpoint_every >= 1");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    if (ctx->forces_pending)
        return fail(JSB_ERR_INVALID_ARGUMENT, "one-shot AddForce cannot be differentiated; use jsb_body_set_step_force");
    if (!ctx->table_host.empty())
        return fail(JSB_ERR_UNSUPPORTED, "differentiable runs use the context's static colliders (no host-determined shapes)");
    for (size_t b = 0; b < ctx->bodies.size(); ++b)
        if (ctx->bodies[b].creation.allow_sleeping)
            return fail(JSB_ERR_UNSUPPORTED, "body " + std::to_string(b) + " may sleep (allow_sleeping), which differentiable runs do not model");
    for (size_t b = 0; b < ctx->bodies.size(); ++b)
        if (!ctx->settings[ctx->bodies[b].settings_id]->parsed.skinned.empty())
            return fail(JSB_ERR_UNSUPPORTED, "body " + std::to_string(b) + " has skinned constraints, which differentiable runs do not model");
    // Reuse the device buffers of the context's previous differentiable run (tape, checkpoints, adjoints):
    // allocating gigabytes of tape costs time every run otherwise.
    auto a = std::make_unique<AdjointSession>();
    if (ctx->adjoint_spare) {
        AdjointSession &o = *ctx->adjoint_spare;
        a->tape_cons = std::move(o.tape_cons);
        a->tape_state = std::move(o.tape_state);
        a->tape_plane = std::move(o.tape_plane);
        a->tape_shape = std::move(o.tape_shape);
        a->tape_cols = std::move(o.tape_cols);
        a->grad_slots = std::move(o.grad_slots);
        a->grad_force = std::move(o.grad_force);
        a->adj_x = std::move(o.adj_x);
        a->adj_v = std::move(o.adj_v);
        a->seed_dev = std::move(o.seed_dev);
        a->final_x = std::move(o.final_x);
        a->final_v = std::move(o.final_v);
        a->final_state = std::move(o.final_state);
        a->ckpt_x = std::move(o.ckpt_x);
        a->ckpt_v = std::move(o.ckpt_v);
        a->ckpt_state = std::move(o.ckpt_state);
        ctx->adjoint_spare.reset();
    }
    a->dt = dt;
    a->steps = num_steps;
    a->every = std::min(checkpoint_every, num_steps);
    const size_t nb = ctx->bodies.size();
    const size_t K = size_t(a->every);
    size_t cons = 0, state = 0, planes = 0, slots = 0;
    std::vector<TapeDesc> desc(nb);
    std::vector<size_t> cons_off(nb), state_off(nb), plane_off(nb);
    a->slot_offset.resize(nb);
    a->step_slots.assign(nb, 0);
    const size_t cap = ctx->max_smem_optin - kStaticSmemReserve;
    for (size_t b = 0; b < nb; ++b) {
        const BodyRec &br = ctx->bodies[b];
        const SettingsRec &s = *ctx->settings[br.settings_id];
        const size_t nv = s.parsed.vertices.size(), ns = s.schedule.num_slots, it = br.creation.num_iterations;
        if (const StepSchedRec *ss = step_sched(ctx, br)) a->step_slots[b] = ss->sched.num_slots;
        cons_off[b] = cons;
        state_off[b] = state;
        plane_off[b] = planes;
        a->slot_offset[b] = slots;
        cons += a->step_slots[b] ? K * a->step_slots[b] * 3 : K * it * ns * 3;
        state += K * it * 3 * nv;
        planes += K * nv;
        slots += a->step_slots[b] ? a->step_slots[b] : ns;
    }
    JSB_CUDA(a->tape_cons.ensure(cons));
    JSB_CUDA(a->tape_state.ensure(state));
    JSB_CUDA(a->tape_plane.ensure(planes));
    JSB_CUDA(a->tape_shape.ensure(planes));
    JSB_CUDA(a->tape_cols.ensure(nb * K * kMaxCollidingShapes));
    JSB_CUDA(a->grad_slots.ensure(std::max<size_t>(slots, 1)));
    JSB_CUDA(a->grad_force.ensure(nb * 3));
    for (size_t b = 0; b < nb; ++b) {
        desc[b].cons = a->tape_cons.ptr + cons_off[b];
        desc[b].state = a->tape_state.ptr + state_off[b];
        desc[b].plane = a->tape_plane.ptr + plane_off[b];
        desc[b].shape = a->tape_shape.ptr + plane_off[b];
        desc[b].cols = a->tape_cols.ptr + b * K * kMaxCollidingShapes;
        desc[b].grad = a->grad_slots.ptr + a->slot_offset[b];
        desc[b].slots = ctx->settings[ctx->bodies[b].settings_id]->schedule.num_slots;
        desc[b].step_slots = a->step_slots[b];
    }
    JSB_CUDA(a->tape_desc.upload(desc.data(), nb));
    JSB_CUDA(a->adj_x.ensure(ctx->total_vertices));
    JSB_CUDA(a->adj_v.ensure(ctx->total_vertices));
    JSB_CUDA(a->seed_dev.ensure(ctx->total_vertices));
    // One taped-forward / adjoint launch per launch group of the forward step.
    int least = 0, greatest = 0;
    JSB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    JSB_CUDA(cudaEventCreateWithFlags(&a->fork, cudaEventDisableTiming));
    const int ng = int(ctx->groups.size());
    for (int gi = 0; gi < ng; ++gi) {
        const LaunchGroup &g = ctx->groups[gi];
        if (g.cluster > 0)
            return fail(JSB_ERR_UNSUPPORTED, "bodies on the thread-block-cluster path cannot take part in a differentiable run");
        a->groups.emplace_back();
        AdjGroup &ag = a->groups.back();
        for (uint32_t b : g.bodies) {
            const BodyRec &br = ctx->bodies[b];
            const SettingsRec &s = *ctx->settings[br.settings_id];
            ag.cap_vertices = std::max(ag.cap_vertices, uint32_t(s.parsed.vertices.size()));
            ag.cap_faces = std::max(ag.cap_faces, pressure_faces(s, br));
            const StepSchedRec *ss = step_sched(ctx, br);
            ag.max_level_slots = std::max(ag.max_level_slots, ss ? ss->sched.max_level_slots : s.schedule.max_level_slots);
        }
        ag.ring_slots = g.ring_slots;  // the ring the bodies' staging chunks were built for
        ag.tape_smem_state = step_smem_bytes(true, ag.cap_vertices, ag.cap_faces, ag.ring_slots) <= cap;
        const size_t tsmem = step_smem_bytes(ag.tape_smem_state, ag.cap_vertices, ag.cap_faces, ag.ring_slots);
        ag.threads = ag.max_level_slots > 192 ? 256 : 128;
        const uint32_t T = uint32_t(ag.threads);
        if (adjoint_smem_bytes(ag.cap_vertices, ag.cap_faces, 0, 1, ag.threads) > cap || tsmem > cap)
            return fail(JSB_ERR_UNSUPPORTED, "a body is too large for the differentiable (taped) path");
        // Deepest adjoint ring (up to 3 levels ahead, up to 4 slots per thread) that fits beside the state.
        ag.adj_rpt = std::max<uint32_t>(1u, std::min<uint32_t>(4u, (ag.max_level_slots + T - 1) / T));
        ag.adj_depth = 3;
        while (ag.adj_depth > 0 && adjoint_smem_bytes(ag.cap_vertices, ag.cap_faces, ag.adj_depth, ag.adj_rpt, ag.threads) > cap) {
            if (ag.adj_rpt > 1)
                --ag.adj_rpt;
            else
                --ag.adj_depth;
        }
        const size_t asmem = adjoint_smem_bytes(ag.cap_vertices, ag.cap_faces, ag.adj_depth, ag.adj_rpt, ag.threads);
        ag.num_work = uint32_t(g.bodies.size());
        ag.tape_grid = int(std::min<size_t>(
            ag.num_work, size_t(std::max(1, step_tape_occupancy(ag.threads, ag.tape_smem_state, tsmem))) * ctx->num_sms));
        ag.adj_grid = int(std::min<size_t>(ag.num_work, size_t(std::max(1, adjoint_occupancy(asmem, ag.threads))) * ctx->num_sms));
        JSB_CUDA(ag.work.upload(g.bodies.data(), g.bodies.size()));
        const int prio = (ng > 1 && greatest != least) ? least + (greatest - least) * gi / (ng - 1) : least;
        JSB_CUDA(cudaStreamCreateWithPriority(&ag.stream, cudaStreamNonBlocking, prio));
        JSB_CUDA(cudaEventCreateWithFlags(&ag.done, cudaEventDisableTiming));
    }
    const int n_ckpt = (num_steps + a->every - 1) / a->every;
    a->ckpt_x.resize(n_ckpt);
    a->ckpt_v.resize(n_ckpt);
    a->ckpt_state.resize(n_ckpt);
    ctx->adjoint = std::move(a);
    return JSB_OK;
}

jsb_status jsb_adjoint_forward(jsb_context *ctx, int until_step) {
    if (!check_ctx(ctx) || !ctx->adjoint) return fail(JSB_ERR_INVALID_ARGUMENT, "no differentiable run (jsb_adjoint_begin)");
    JSB_CUDA(cudaSetDevice(ctx->device));
    AdjointSession &a = *ctx->adjoint;
    if (until_step < 0) until_step = a.steps;
    if (until_step < a.cur_step || until_step > a.steps)
        return fail(JSB_ERR_INVALID_ARGUMENT, "until_step must lie between the steps already run and num_steps");
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    if (a.cur_step == 0) {
        a.seeds.clear();
        a.backward_done = false;
        a.tape_segment = -1;
    }
    uint32_t launches = 0;
    const int last_seg_start = ((a.steps - 1) / a.every) * a.every;
    if (a.cur_step == 0) a.forward_ms = 0.0f;
    PhaseTimer timer;  // per step: start, end (the checkpoint copies between steps are not counted)
    for (int s = a.cur_step; s < until_step; ++s) {
        if (s % a.every == 0) {
            JSB_CUDA(cudaDeviceSynchronize());
            if ((st = save_state(ctx, a.ckpt_x[s / a.every], a.ckpt_v[s / a.every], a.ckpt_state[s / a.every])) != JSB_OK) return st;
        }
        JSB_CUDA(timer.mark());
        if (s >= last_seg_start) {
            // The last segment runs taped, so the backward pass starts without recomputing it.
            if ((st = enqueue_taped(ctx, a, s - last_seg_start, 0, launches)) != JSB_OK) return st;
        } else if ((st = enqueue_batched(ctx, a.dt, 0, launches)) != JSB_OK)
            return st;
        JSB_CUDA(timer.mark());
    }
    JSB_CUDA(cudaDeviceSynchronize());
    for (size_t k = 0; k + 1 < timer.ev.size(); k += 2) a.forward_ms += timer.between(k, k + 1);
    a.cur_step = until_step;
    if (a.cur_step == a.steps) {
        if ((st = save_state(ctx, a.final_x, a.final_v, a.final_state)) != JSB_OK) return st;
        a.forward_done = true;
        a.tape_segment = (a.steps - 1) / a.every;
    }
    ctx->last_launches = launches;
    return JSB_OK;
}

jsb_status jsb_adjoint_seed(jsb_context *ctx, int step, uint32_t body_id, const float *dl_dx) {
    if (!check_ctx(ctx) || !ctx->adjoint || !dl_dx || body_id >= ctx->bodies.size())
        return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    AdjointSession &a = *ctx->adjoint;
    if (step < 1 || step > a.steps) return fail(JSB_ERR_INVALID_ARGUMENT, "seed step must be in 1 .. num_steps");
    std::vector<float4> *dst = nullptr;
    for (auto &sd : a.seeds)
        if (sd.first == step) dst = &sd.second;
    if (!dst) {
        a.seeds.push_back({step, std::vector<float4>(ctx->total_vertices, make_float4(0, 0, 0, 0))});
        dst = &a.seeds.back().second;
    }
    const BodyRec &b = ctx->bodies[body_id];
    const size_t nv = ctx->settings[b.settings_id]->parsed.vertices.size();
    for (size_t i = 0; i < nv; ++i) {
        float4 &d = (*dst)[b.vtx_offset + i];
        d.x += dl_dx[3 * i + 0];
        d.y += dl_dx[3 * i + 1];
        d.z += dl_dx[3 * i + 2];
    }
    return JSB_OK;
}

jsb_status jsb_adjoint_seed_all(jsb_context *ctx, int step, const float *dl_dx) {
    if (!check_ctx(ctx) || !ctx->adjoint || !dl_dx) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    AdjointSession &a = *ctx->adjoint;
    if (step < 1 || step > a.steps) return fail(JSB_ERR_INVALID_ARGUMENT, "seed step must be in 1 .. num_steps");
    std::vector<float4> *dst = nullptr;
    for (auto &sd : a.seeds)
        if (sd.first == step) dst = &sd.second;
    if (!dst) {
        a.seeds.push_back({step, std::vector<float4>(ctx->total_vertices, make_float4(0, 0, 0, 0))});
        dst = &a.seeds.back().second;
    }
    for (uint64_t i = 0; i < ctx->total_vertices; ++i) {
        float4 &d = (*dst)[i];
        d.x += dl_dx[3 * i + 0];
        d.y += dl_dx[3 * i + 1];
        d.z += dl_dx[3 * i + 2];
    }
    return JSB_OK;
}

jsb_status jsb_adjoint_gradients_all(jsb_context *ctx, float *dl_dx0, float *dl_dv0, float *dl_dforce) {
    if (!check_ctx(ctx) || !ctx->adjoint) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    AdjointSession &a = *ctx->adjoint;
    if (!a.backward_done) return fail(JSB_ERR_INVALID_ARGUMENT, "jsb_adjoint_backward has not run");
    JSB_CUDA(cudaSetDevice(ctx->device));
    const uint64_t n = ctx->total_vertices;
    std::vector<float4> tmp(n);
    float *outs[2] = {dl_dx0, dl_dv0};
    const DevBuf<float4> *srcs[2] = {&a.adj_x, &a.adj_v};
    for (int k = 0; k < 2; ++k) {
        if (!outs[k]) continue;
        JSB_CUDA(cudaMemcpy(tmp.data(), srcs[k]->ptr, n * sizeof(float4), cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < n; ++i) {
            outs[k][3 * i + 0] = tmp[i].x;
            outs[k][3 * i + 1] = tmp[i].y;
            outs[k][3 * i + 2] = tmp[i].z;
        }
    }
    if (dl_dforce && !ctx->bodies.empty())
        JSB_CUDA(cudaMemcpy(dl_dforce, a.grad_force.ptr, ctx->bodies.size() * 3 * sizeof(float), cudaMemcpyDeviceToHost));
    return JSB_OK;
}

jsb_status jsb_adjoint_backward(jsb_context *ctx) {
    if (!check_ctx(ctx) || !ctx->adjoint) return fail(JSB_ERR_INVALID_ARGUMENT, "no differentiable run (jsb_adjoint_begin)");
    AdjointSession &a = *ctx->adjoint;
    if (!a.forward_done) return fail(JSB_ERR_INVALID_ARGUMENT, "jsb_adjoint_forward must run before the backward pass");
    JSB_CUDA(cudaSetDevice(ctx->device));
    jsb_status st = rebuild(ctx);
    if (st != JSB_OK) return st;
    const uint64_t n = ctx->total_vertices;
    JSB_CUDA(cudaMemset(a.adj_x.ptr, 0, n * sizeof(float4)));
    JSB_CUDA(cudaMemset(a.adj_v.ptr, 0, n * sizeof(float4)));
    JSB_CUDA(cudaMemset(a.grad_slots.ptr, 0, a.grad_slots.count * sizeof(float)));
    JSB_CUDA(cudaMemset(a.grad_force.ptr, 0, a.grad_force.count * sizeof(float)));
    uint32_t launches = 0;
    const int n_ckpt = int(a.ckpt_x.size());
    PhaseTimer timer;  // per segment: recompute start / end, reverse end
    for (int seg = n_ckpt - 1; seg >= 0; --seg) {
        const int s0 = seg * a.every, s1 = std::min(s0 + a.every, a.steps);
        JSB_CUDA(timer.mark());
        if (a.tape_segment != seg) {  // the forward pass leaves the last segment's tape in place
            if ((st = load_state(ctx, a.ckpt_x[seg], a.ckpt_v[seg], a.ckpt_state[seg])) != JSB_OK) return st;
            for (int s = s0; s < s1; ++s)  // recompute the segment, recording the tape
                if ((st = enqueue_taped(ctx, a, s - s0, 0, launches)) != JSB_OK) return st;
            a.tape_segment = seg;
        }
        JSB_CUDA(timer.mark());
        for (int s = s1 - 1; s >= s0; --s) {  // reverse the segment
            for (auto &sd : a.seeds)
                if (sd.first == s + 1) {
                    JSB_CUDA(cudaMemcpy(a.seed_dev.ptr, sd.second.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
                    JSB_CUDA(launch_add(a.adj_x.ptr, a.seed_dev.ptr, n, ctx->num_sms, 0));
                    ++launches;
                }
            if ((st = enqueue_adjoint(ctx, a, s - s0, 0, launches)) != JSB_OK) return st;
        }
        JSB_CUDA(timer.mark());
    }
    JSB_CUDA(cudaDeviceSynchronize());
    a.recompute_ms = a.reverse_ms = 0.0f;
    for (size_t k = 0; k + 2 < timer.ev.size() + 1; k += 3) {
        a.recompute_ms += timer.between(k, k + 1);
        a.reverse_ms += timer.between(k + 1, k + 2);
    }
    if ((st = load_state(ctx, a.final_x, a.final_v, a.final_state)) != JSB_OK) return st;
    a.backward_done = true;
    ctx->last_launches = launches;
    return JSB_OK;
}

jsb_status jsb_adjoint_gradients(jsb_context *ctx, uint32_t body_id, float *dl_dx0, float *dl_dv0, float *dl_dforce,
                                 float *dl_dedge_compliance, float *dl_dvolume_compliance) {
    if (!check_ctx(ctx) || !ctx->adjoint || body_id >= ctx->bodies.size()) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument");
    AdjointSession &a = *ctx->adjoint;
    if (!a.backward_done) return fail(JSB_ERR_INVALID_ARGUMENT, "jsb_adjoint_backward has not run");
    JSB_CUDA(cudaSetDevice(ctx->device));
    const BodyRec &b = ctx->bodies[body_id];
    const SettingsRec &s = *ctx->settings[b.settings_id];
    const size_t nv = s.parsed.vertices.size();
    std::vector<float4> tmp(nv);
    if (dl_dx0) {
        JSB_CUDA(cudaMemcpy(tmp.data(), a.adj_x.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nv; ++i) {
            dl_dx0[3 * i + 0] = tmp[i].x;
            dl_dx0[3 * i + 1] = tmp[i].y;
            dl_dx0[3 * i + 2] = tmp[i].z;
        }
    }
    if (dl_dv0) {
        JSB_CUDA(cudaMemcpy(tmp.data(), a.adj_v.ptr + b.vtx_offset, nv * sizeof(float4), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nv; ++i) {
            dl_dv0[3 * i + 0] = tmp[i].x;
            dl_dv0[3 * i + 1] = tmp[i].y;
            dl_dv0[3 * i + 2] = tmp[i].z;
        }
    }
    if (dl_dforce) JSB_CUDA(cudaMemcpy(dl_dforce, a.grad_force.ptr + 3 * body_id, 3 * sizeof(float), cudaMemcpyDeviceToHost));
    if (dl_dedge_compliance || dl_dvolume_compliance) {
        // per-slot sums of the reverse sweep -> Jolt's constraint order (a whole-step schedule holds each
        // constraint once per substep)
        const uint32_t step_slots = a.step_slots[body_id];
        StepSchedule steps;
        if (step_slots && (!build_step_schedule(s.parsed, b.creation.num_iterations, steps, true) || steps.num_slots != step_slots))
            return fail(JSB_ERR_CAPACITY, "whole-step schedule rebuild failed");
        const std::vector<uint32_t> &source = step_slots ? steps.source : s.schedule.padded_source;
        const size_t stride = step_slots ? 2 : 1;
        std::vector<float> g(step_slots ? step_slots : s.schedule.num_slots);
        if (!g.empty())
            JSB_CUDA(cudaMemcpy(g.data(), a.grad_slots.ptr + a.slot_offset[body_id], g.size() * sizeof(float), cudaMemcpyDeviceToHost));
        if (dl_dedge_compliance) std::fill(dl_dedge_compliance, dl_dedge_compliance + s.parsed.edges.size(), 0.0f);
        if (dl_dvolume_compliance) std::fill(dl_dvolume_compliance, dl_dvolume_compliance + s.parsed.volumes.size(), 0.0f);
        for (size_t c = 0; c < g.size(); ++c) {
            const uint32_t src = source[c * stride];
            if (src == 0xffffffffu) continue;
            const uint32_t type = src >> 28, idx = src & 0x0fffffffu;
            if (type == kEdge && dl_dedge_compliance) dl_dedge_compliance[idx] += g[c];
            if (type == kVolume && dl_dvolume_compliance) dl_dvolume_compliance[idx] += g[c];
        }
    }
    return JSB_OK;
}

jsb_status jsb_adjoint_timings(jsb_context *ctx, float out_ms[3]) {
    if (!check_ctx(ctx) || !ctx->adjoint || !out_ms) return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument or no differentiable run");
    out_ms[0] = ctx->adjoint->forward_ms;
    out_ms[1] = ctx->adjoint->recompute_ms;
    out_ms[2] = ctx->adjoint->reverse_ms;
    return JSB_OK;
}

jsb_status jsb_adjoint_bend_gradients(jsb_context *ctx, uint32_t body_id, float *dl_dbend_compliance) {
    if (!check_ctx(ctx) || !ctx->adjoint || body_id >= ctx->bodies.size() || !dl_dbend_compliance)
        return fail(JSB_ERR_INVALID_ARGUMENT, "bad argument or no differentiable run");
    AdjointSession &a = *ctx->adjoint;
    if (!a.backward_done) return fail(JSB_ERR_INVALID_ARGUMENT, "jsb_adjoint_backward has not run");
    JSB_CUDA(cudaSetDevice(ctx->device));
    JSB_CUDA(cudaDeviceSynchronize());
    const BodyRec &b = ctx->bodies[body_id];
    const SettingsRec &s = *ctx->settings[b.settings_id];
    const uint32_t step_slots = a.step_slots[body_id];
    StepSchedule steps;
    if (step_slots && (!build_step_schedule(s.parsed, b.creation.num_iterations, steps, true) || steps.num_slots != step_slots))
        return fail(JSB_ERR_CAPACITY, "whole-step schedule rebuild failed");
    const std::vector<uint32_t> &source = step_slots ? steps.source : s.schedule.padded_source;
    const size_t stride = step_slots ? 2 : 1;
    std::vector<float> g(step_slots ? step_slots : s.schedule.num_slots);
    if (!g.empty())
        JSB_CUDA(cudaMemcpy(g.data(), a.grad_slots.ptr + a.slot_offset[body_id], g.size() * sizeof(float), cudaMemcpyDeviceToHost));
    std::fill(dl_dbend_compliance, dl_dbend_compliance + s.parsed.bends.size(), 0.0f);
    for (size_t c = 0; c < g.size(); ++c) {
        const uint32_t src = source[c * stride];
        if (src != 0xffffffffu && (src >> 28) == kBend) dl_dbend_compliance[src & 0x0fffffffu] += g[c];
    }
    return JSB_OK;
}

jsb_status jsb_adjoint_end(jsb_context *ctx) {
    if (!check_ctx(ctx)) return JSB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    if (ctx->adjoint) {  // keep the device buffers for the next differentiable run of this context
        ctx->adjoint->release_launch_groups();
        ctx->adjoint_spare = std::move(ctx->adjoint);
    }
    return JSB_OK;
}

}  // extern "C"
