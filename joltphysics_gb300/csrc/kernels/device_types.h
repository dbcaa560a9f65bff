// Data layout shared by the host runtime and the CUDA kernels.
//
// HBM layout of one context:
//   vertex state, SoA over all bodies (body b owns [vtx_offset, vtx_offset + num_vertices)):
//     x      float4  position (local to the body) in xyz, inverse mass in w
//     v      float4  velocity in xyz
//   per-step scratch, same indexing:
//     prev   float4  position before the current substep's integration
//     plane  float4  collision plane (normal xyz, constant w), relative to the body
//     shape  int32   index into the body's colliding-shape list, -1 = none
//   per settings object (shared by all bodies created from it):
//     levels  uint4[num_levels + 2]  {first record, end of bends, end of volumes, end of edges};
//                                    the LRA records of level l end where level l + 1 starts
//     records uint4[num_records]     16-byte constraint records in dependency-level order
//     faces   uint4[num_faces]       {v0, v1, v2, 0} (pressure only)
//     vf_off  uint32[num_vertices+1] incident faces of each vertex, ascending (pressure only)
//     vf      uint32[...]
// Constraint records (vertex indices are 16-bit, local to the body):
//   bend   {v0 | v1 << 16, v2 | v3 << 16, compliance, initial angle}
//   volume {v0 | v1 << 16, v2 | v3 << 16, six rest volume, compliance}
//   edge   {v0 | v1 << 16, 0, rest length, compliance}
//   LRA    {v0 | v1 << 16, 0, max distance, 0}
//   per (settings, iteration count), bodies without pressure:
//     step_levels  uint4[num_step_levels]  whole-step dependency levels (host/schedule.h)
//     step_records uint4[...]              the step's constraint records and per-vertex slots
#pragma once

#include <stdint.h>
#include <vector_types.h>

#if defined(__CUDACC__)
#define JSB_HD __host__ __device__
#else
#define JSB_HD
#endif

namespace jsb {

constexpr uint32_t kMaxVerticesPerBody = 65536;
constexpr uint32_t kStageLevels = 64;  // level descriptors per schedule-ring half (the per-substep walk stages one more)
constexpr uint32_t kMaxCollidingShapes = 16;  // colliding shapes kept per body per step

enum : uint32_t { kFlagUpdatePosition = 1u, kFlagAllowSleeping = 2u };

// Device error word bits.
enum : uint32_t { kErrNonFinite = 1u, kErrShapeOverflow = 2u, kErrTimeout = 4u };

struct BodyDesc {
    // shared settings
    const uint4 *levels;
    const uint4 *records;
    const uint4 *faces;
    const uint32_t *vf_off;
    const uint32_t *vf;
    uint32_t num_levels;
    uint32_t num_records;
    uint32_t num_faces;
    uint32_t num_vertices;
    // whole-step schedule for this body's iteration count (null: walk the per-substep schedule);
    // levels {first slot, bend end | volume end << 16, edge end | LRA end << 16, slots}, vertex slots
    // {vertex index, substep entered, 0, 0} from the LRA end on (see build_step_schedule)
    const uint4 *step_levels;
    const uint4 *step_records;
    uint32_t num_step_levels;
    // staging chunks of the two schedules (host/schedule.h build_stage_chunks) for ring halves of
    // stage_half record slots: {first level, end level, first slot, staged slots}
    const uint4 *chunks;
    const uint4 *step_chunks;
    uint32_t num_chunks;
    uint32_t num_step_chunks;
    uint32_t stage_half;
    // body
    uint32_t vtx_offset;
    uint32_t num_iterations;
    float linear_damping;
    float max_linear_velocity;
    float restitution;
    float friction;
    float pressure;
    float gravity_factor;
    float vertex_radius;
    uint32_t flags;
    // skinned constraints (null: none): per constraint {max distance, back stop distance, back stop radius,
    // vertex}; per vertex of the body three float4 {previous position, position, normal}
    // (SoftBodyMotionProperties::SkinState)
    const float4 *skin_params;
    float4 *skin_state;
    float4 *face_scratch;  // pressure on the cluster path: one float4 per face (null: none)
};

// Run-time skinning switches of one body (SoftBodyMotionProperties::mEnableSkinConstraints,
// mSkinnedMaxDistanceMultiplier, mSkinStatePreviousPositionValid).
struct SkinCtl {
    float max_distance_multiplier;
    uint32_t flags;  // kSkinEnabled | kSkinPreviousValid
};
enum : uint32_t { kSkinEnabled = 1, kSkinPreviousValid = 2 };

enum : int32_t { kMotionStatic = 0, kMotionKinematic = 1, kMotionDynamic = 2 };  // EMotionType
constexpr int32_t kMotionSensor = 3;  // a leaf shape of a sensor (SoftBodyMotionProperties::CollidingSensor)

// A colliding shape of one body determined on the host (jsb_colliding_shape as uploaded): the fields of
// SoftBodyMotionProperties::CollidingShape and its LeafShape that the step reads.
struct ShapeEntry {
    int32_t type, motion;
    float xf[12];  // leaf transform relative to the soft body: rotation columns 0-2, then translation
    float half_extent[3], radius, friction, restitution;
    float inv_mass_scale;   // mSoftBodyInvMassScale
    float inv_mass;         // dynamic: mInvMass
    float inv_inertia[12];  // dynamic: mInvInertia, columns 0-3
    float com[3];           // mCenterOfMassTransform translation
    float lin[3], ang[3];   // dynamic: velocities at the start of the step (soft-body space)
    uint32_t hull;          // convex hulls: index into StepParams::hulls
};

// A registered convex hull (jsb_hull_add): planes then points as float4 from `f4` (StepParams::hull_f4),
// each face's first vertex and vertex count {first, count} from `faces`, vertex indices from `indices`
// (StepParams::hull_u32).
struct HullDev {
    uint32_t num_faces, num_points;
    uint32_t f4;       // planes at [f4, f4 + num_faces), points at [f4 + num_faces, ... + num_points)
    uint32_t faces;    // {first, count} pairs at [faces, faces + 2 num_faces) in hull_u32
};

// Per body with host-determined colliding shapes: the shapes, and after a step the dynamic shapes'
// velocities (mLinearVelocity / mAngularVelocity) and which of them a contact changed (mUpdateVelocities).
struct ShapeTable {
    uint32_t count;
    uint32_t updated;  // bit s: shape s
    uint32_t pad[2];
    ShapeEntry e[kMaxCollidingShapes];
    float lin[kMaxCollidingShapes][4];
    float ang[kMaxCollidingShapes][4];
};

struct BodyState {
    float position[3];  // body position in world space
    float bmin[3], bmax[3];  // local bounds
    float pmin[3], pmax[3];  // local predicted bounds
    float lin_vel[3], ang_vel[3];
};

// Sleep state of a body (MotionProperties::mSleepTestTimer and whether the body is in the active set).
struct BodySleep {
    float timer;
    uint32_t active;  // 0: asleep, not stepped until a force or jsb_body_activate wakes it
};

struct ColliderDev {
    int32_t type;  // 0 box, 1 sphere
    float position[3];
    float half_extent[3];
    float radius;
    float friction;
    float restitution;
};

// Per-body tape of one checkpoint segment of a differentiable run (written by the taped forward step,
// read by the adjoint step).
struct TapeDesc {
    float4 *cons;    // [segment substeps][slots][3]: constraint inputs as vertex differences
    float4 *state;   // [segment substeps][3][num_vertices]: x at substep start, v after integration,
                     //                                     x after the constraint levels
    float4 *plane;   // [segment steps][num_vertices]: collision plane (normal, constant)
    int32_t *shape;  // [segment steps][num_vertices]: colliding shape index, -1 none
    float2 *cols;    // [segment steps][kMaxCollidingShapes]: combined friction, restitution
    float *grad;     // [slots] (or [step_slots]): d loss / d compliance of the slot's constraint
    uint32_t slots;       // slots of the per-substep schedule
    uint32_t step_slots;  // > 0: the body walks its whole-step schedule of this many slots; cons is then
                          // [segment steps][step_slots][3] and grad [step_slots]
};

// Slot type of a whole-step level {first, bend end | volume end << 16, edge end | LRA end << 16, slots}:
// 0 bend, 1 volume, 2 edge, 3 LRA, 4 vertex.
JSB_HD inline int step_slot_type(uint4 lv, uint32_t s) {
    return s < (lv.y & 0xffffu) ? 0 : (s < (lv.y >> 16) ? 1 : (s < (lv.z & 0xffffu) ? 2 : (s < (lv.z >> 16) ? 3 : 4)));
}

struct StepParams {
    const BodyDesc *bodies;
    BodyState *states;
    const uint32_t *work;  // body indices, most expensive first
    uint32_t num_work;
    uint32_t *queue;  // work queue counter (zeroed before each launch)
    float4 *x;
    float4 *v;
    float4 *prev;
    float4 *plane;
    int32_t *shape;
    const ColliderDev *colliders;
    uint32_t num_colliders;
    float gravity[3];
    float dt;
    uint32_t *error;
    const float *forces;  // 3 floats per body: AddForce accumulators consumed by this step
    const float *step_forces;  // 3 floats per body: force added before every step (persistent)
    uint32_t ring_slots;  // record slots per schedule-ring half (>= every launched body's stage_half)
    const TapeDesc *tape;  // per-body tapes (taped forward only)
    uint32_t tape_step;    // step index within the checkpoint segment (taped forward only)
    ShapeTable *tables;        // host-determined colliding shapes (null: none)
    const int32_t *table_slot; // per body: index into tables, -1 = the context's colliders
    int32_t *dyn_list;         // per vertex (context indexing): scratch for the vertices touching dynamic shapes
    uint8_t *contact;          // per vertex (null: not recorded): touched its collision plane this step (mHasContact)
    float4 *contact_point;     // per vertex: SoftBodyManifold::GetLocalContactPoint (before the recentring)
    float *contact_delta;      // 3 per body: the recentring offset of the step
    const HullDev *hulls;      // registered convex hulls
    const float4 *hull_f4;
    const uint32_t *hull_u32;
    uint32_t *sensor_contact;  // per body: bit k = sensor shape k of its table has a vertex inside it (mHasContact)
    SkinCtl *skin_ctl;         // per body
    BodySleep *sleep;      // per body (null: bodies never sleep)
    float sleep_velocity_threshold;  // PhysicsSettings::mPointVelocitySleepThreshold (compared with |v|^2)
    float time_before_sleep;         // PhysicsSettings::mTimeBeforeSleep
};

// Parameters of one adjoint step over a set of bodies (the reverse of one forward step).
struct AdjParams {
    const BodyDesc *bodies;
    const TapeDesc *tape;
    uint32_t tape_step;  // step index within the checkpoint segment
    const uint32_t *work;
    uint32_t num_work;
    uint32_t *queue;
    float4 *adj_x;  // d loss / d position (local = world), context vertex indexing
    float4 *adj_v;  // d loss / d velocity
    float *grad_force;  // 3 per body
    float gravity[3];
    float dt;
    uint32_t ring_depth;  // levels of records + taped inputs streamed ahead (0: read in place)
    uint32_t ring_rpt;    // ring slots per thread and level
};

}  // namespace jsb
