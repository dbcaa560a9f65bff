/*
 * jsb: GB300-native soft-body solver step for Jolt Physics, C ABI.
 *
 * This is the drop-in boundary for SoftBodyMotionProperties' update
 * (Jolt/Physics/SoftBody/SoftBodyMotionProperties.cpp:937-1256). A Jolt integration keeps building
 * SoftBodySharedSettings / SoftBodyCreationSettings with Jolt, passes the settings bytes written by
 * SoftBodySharedSettings::SaveBinaryState (SoftBodySharedSettings.cpp:1203-1236) and, optionally, the
 * per-body state written by SoftBodyMotionProperties::SaveState (SoftBodyMotionProperties.cpp:1446-1473),
 * steps bodies on the GPU and reads state back in the RestoreState layout (:1475-1502) together with
 * the body position delta that PhysicsSystem::JobSoftBodyFinalize applies (PhysicsSystem.cpp:2864).
 *
 * Conventions: every call returns a jsb_status (0 = JSB_OK); no C++ exception crosses the boundary;
 * jsb_last_error_string() describes the last failure of the calling thread. A context belongs to one
 * host thread. Calls that take a stream enqueue work on it; calls without one synchronise.
 * All pointers are host pointers unless the name says "device".
 */
#ifndef JSB_H
#define JSB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int jsb_status;
enum {
    JSB_OK = 0,
    JSB_ERR_INVALID_ARGUMENT = 1, /* null pointer, unknown id, bad size */
    JSB_ERR_BLOB = 2,             /* malformed settings/state bytes (truncated, out-of-range index) */
    JSB_ERR_UNSUPPORTED = 3,      /* constraint type or body size the GPU path does not handle */
    JSB_ERR_CUDA = 4,             /* a CUDA runtime call failed */
    JSB_ERR_OUT_OF_MEMORY = 5,    /* device allocation failed */
    JSB_ERR_TIMEOUT = 6,          /* a bounded device wait gave up */
    JSB_ERR_NONFINITE = 7,        /* a NaN/Inf vertex position or velocity was produced */
    JSB_ERR_CAPACITY = 8          /* a fixed-size limit was exceeded */
};

typedef struct jsb_context jsb_context;
typedef struct CUstream_st *jsb_stream; /* cudaStream_t; NULL = the default stream */

/* SoftBodyCreationSettings scalars (Jolt/Physics/SoftBody/SoftBodyCreationSettings.h:61-72). */
typedef struct jsb_creation_settings {
    uint32_t num_iterations;      /* mNumIterations */
    float linear_damping;         /* mLinearDamping */
    float max_linear_velocity;    /* mMaxLinearVelocity */
    float restitution;            /* mRestitution */
    float friction;               /* mFriction */
    float pressure;               /* mPressure */
    float gravity_factor;         /* mGravityFactor */
    float vertex_radius;          /* mVertexRadius */
    uint8_t update_position;      /* mUpdatePosition */
    uint8_t make_rotation_identity; /* mMakeRotationIdentity (must be 1: bodies keep identity rotation) */
    uint8_t allow_sleeping;       /* mAllowSleeping: the body may fall asleep (see jsb_set_sleep_settings) */
    uint8_t faces_double_sided;   /* mFacesDoubleSided (queries only) */
} jsb_creation_settings;

enum { JSB_COLLIDER_BOX = 0, JSB_COLLIDER_SPHERE = 1, JSB_COLLIDER_CAPSULE = 2, JSB_COLLIDER_CYLINDER = 3, JSB_COLLIDER_HULL = 4 };

/* A static rigid body with one convex leaf shape (BoxShape / SphereShape / CapsuleShape / CylinderShape),
 * world space, identity rotation (capsules and cylinders along the Y axis). friction/restitution are the
 * body's; they are combined with the soft body's like ContactConstraintManager's defaults (sqrt(f1 f2),
 * max(r1, r2)). */
typedef struct jsb_collider {
    int32_t type;         /* JSB_COLLIDER_* */
    float position[3];
    float half_extent[3]; /* box: half extents; capsule: [1] = half height of the cylinder part
                             (CapsuleShape's inHalfHeightOfCylinder); cylinder: [1] = half height */
    float radius;         /* sphere, capsule, cylinder */
    float friction;
    float restitution;
} jsb_collider;

/* ---- context ------------------------------------------------------------------------------ */
jsb_status jsb_context_create(int device, jsb_context **out);
jsb_status jsb_context_destroy(jsb_context *ctx);
const char *jsb_last_error_string(void);
const char *jsb_version(void);

/* PhysicsSystem::SetGravity (PhysicsSystem.h). */
jsb_status jsb_set_gravity(jsb_context *ctx, const float gravity[3]);

/* ---- settings and bodies ------------------------------------------------------------------ */
/* Upload SoftBodySharedSettings::SaveBinaryState bytes (SoftBodySharedSettings.cpp:1203-1236).
 * Settings are immutable and may be shared by many bodies. Rejects skinned constraints and rods
 * (JSB_ERR_UNSUPPORTED) and bodies with more than 65536 vertices. */
jsb_status jsb_settings_upload(jsb_context *ctx, const void *blob, size_t len, uint32_t *settings_id);

/* BodyInterface::CreateSoftBody + SoftBodyMotionProperties::Initialize (SoftBodyMotionProperties.cpp:59-105):
 * vertices start at the settings' positions/velocities. `position` is the body position in world space. */
jsb_status jsb_body_add(jsb_context *ctx, uint32_t settings_id, const jsb_creation_settings *creation,
                        const float position[3], uint32_t *body_id);

/* Overwrite a body's state with SoftBodyMotionProperties::SaveState bytes (single precision build,
 * no rods/skinning: 101-byte MotionProperties header, N x (position, velocity), 4 bounds vectors). */
jsb_status jsb_body_restore_state(jsb_context *ctx, uint32_t body_id, const void *state, size_t len,
                                  const float position[3]);

/* MotionProperties::AddForce: accumulated until the next step consumes it (ResetForce). */
jsb_status jsb_body_add_force(jsb_context *ctx, uint32_t body_id, const float force[3]);

/* A force added before every step (the effect of calling AddForce with the same value before each
 * PhysicsSystem::Update); kept until changed. Unlike jsb_body_add_force it can be captured in graphs. */
jsb_status jsb_body_set_step_force(jsb_context *ctx, uint32_t body_id, const float force[3]);

jsb_status jsb_collider_add(jsb_context *ctx, const jsb_collider *collider, uint32_t *collider_id);

/* Sleeping (SoftBodyMotionProperties.cpp:902-915, PhysicsSystem.cpp:2875-2884): after each step a body
 * created with allow_sleeping whose largest squared vertex velocity (before the velocity clamp) is at or
 * below point_velocity_sleep_threshold adds the step's dt to its sleep timer, else restarts it; once the
 * timer reaches time_before_sleep the body goes to sleep: it is no longer stepped and its body velocities
 * read zero. A force (jsb_body_add_force, or a non-zero jsb_body_set_step_force before every step) wakes
 * it and restarts its timer, as BodyInterface::AddForce does. PhysicsSettings::mTimeBeforeSleep /
 * mPointVelocitySleepThreshold (PhysicsSettings.h:95,102); defaults 0.5 s and 0.03 (m/s)^2. */
jsb_status jsb_set_sleep_settings(jsb_context *ctx, float time_before_sleep, float point_velocity_sleep_threshold);
/* BodyInterface::IsActive / ActivateBody (restarts the sleep timer) / DeactivateBody. */
jsb_status jsb_body_is_active(jsb_context *ctx, uint32_t body_id, int *active);
jsb_status jsb_body_set_active(jsb_context *ctx, uint32_t body_id, int active);

jsb_status jsb_body_num_vertices(jsb_context *ctx, uint32_t body_id, uint32_t *num_vertices);

/* ---- host-determined colliding shapes (rigid bodies that move; two-way coupling) ------------- */
enum { JSB_MOTION_STATIC = 0, JSB_MOTION_KINEMATIC = 1, JSB_MOTION_DYNAMIC = 2 }; /* EMotionType */
/* A leaf shape of a sensor (SoftBodyMotionProperties::CollidingSensor, collected when the contact listener
 * accepts a body with SoftBodyContactSettings::mIsSensor: SoftBodyMotionProperties.cpp:191-198): it moves
 * no vertex; the step reports whether a vertex with inverse mass > 0 penetrates it (jsb_body_sensor_contacts). */
enum { JSB_MOTION_SENSOR = 3 };

/* One colliding shape of a soft body, as SoftBodyMotionProperties::DetermineCollidingShapes collects it
 * (SoftBodyMotionProperties.cpp:120-255; fields of CollidingShape and its LeafShape, SoftBodyMotionProperties.h):
 * the adapter fills it from the same values inside PhysicsSystem's soft-body prepare job. Matrices are
 * Jolt's Mat44 columns, xyz of each. */
typedef struct jsb_colliding_shape {
    int32_t type;             /* JSB_COLLIDER_*: the leaf shape (Box / Sphere / Capsule / Cylinder / ConvexHull) */
    int32_t motion_type;      /* JSB_MOTION_*: CollidingShape::mMotionType */
    float transform[12];      /* LeafShape::mTransform (relative to the soft body): rotation columns 0-2, translation */
    float half_extent[3];     /* box; [1] = half height of a capsule's cylinder part / a cylinder */
    float radius;             /* sphere, capsule, cylinder */
    float friction;           /* CollidingShape::mFriction (combined) */
    float restitution;        /* CollidingShape::mRestitution (combined) */
    float soft_body_inv_mass_scale; /* mSoftBodyInvMassScale (1 unless a contact listener changed it) */
    float inv_mass;           /* dynamic: mInvMass */
    float inv_inertia[12];    /* dynamic: mInvInertia, columns 0-3 */
    float center_of_mass[3];  /* mCenterOfMassTransform's translation */
    float linear_velocity[3]; /* dynamic: mLinearVelocity at the start of the step (soft-body space) */
    float angular_velocity[3];/* dynamic: mAngularVelocity */
    uint32_t hull_id;         /* JSB_COLLIDER_HULL: the id jsb_hull_add returned */
} jsb_colliding_shape;

/* A ConvexHullShape as Jolt built it (host-determined shapes only): its points relative to the shape's
 * centre of mass (GetPoint), one plane per face (GetPlanes: normal xyz, constant) and each face's vertex
 * indices (GetFaceVertices), at most 256 points and 255 faces. CollideSoftBodyVertices of an unscaled hull
 * (ConvexHullShape.cpp:1060-1163) then runs on the GPU. Hulls are registered once and used by id. */
typedef struct jsb_convex_hull {
    uint32_t num_points;
    const float *points;                /* 3 per point */
    uint32_t num_faces;
    const float *planes;                /* 4 per face */
    const uint32_t *face_vertex_counts; /* per face */
    const uint32_t *face_vertices;      /* the faces' vertex indices, concatenated */
} jsb_convex_hull;
jsb_status jsb_hull_add(jsb_context *ctx, const jsb_convex_hull *hull, uint32_t *hull_id);

/* Replaces the context's static colliders for one body with `count` (<= 16) host-determined shapes, in
 * the order the reference collects them; they apply to every following step (each of its collision
 * steps) until set again or cleared. Vertices on a dynamic shape take the dynamic-body branch of
 * ApplyCollisionConstraintsAndUpdateVelocities (:752-797) in vertex order, such bodies walk their schedule
 * substep by substep, and the shape's velocities change with each impulse. Taken on the one-CTA and the
 * thread-block-cluster paths; not for graphs (jsb_step_graph) or differentiable runs (JSB_ERR_UNSUPPORTED). */
jsb_status jsb_body_set_colliding_shapes(jsb_context *ctx, uint32_t body_id, const jsb_colliding_shape *shapes, uint32_t count);
jsb_status jsb_body_clear_colliding_shapes(jsb_context *ctx, uint32_t body_id);
/* After a step (synchronises the device): per host-determined shape of the body, 7 floats {updated (1 when a
 * contact changed the shape's velocities: CollidingShape::mUpdateVelocities), linear velocity[3], angular
 * velocity[3]} in soft-body space; *count = the number of shapes. UpdateRigidBodyVelocities (:923-935) then
 * adds the soft body's rotation times (velocity - the shape's input velocity) to the rigid body. */
jsb_status jsb_body_shape_velocities(jsb_context *ctx, uint32_t body_id, float *out, uint32_t *count);

/* ---- contacts (SoftBodyManifold) ---------------------------------------------------------------- */
/* Records, every step, what SoftBodyManifold exposes to ContactListener::OnSoftBodyContactAdded
 * (SoftBodyManifold.h; SoftBodyMotionProperties.cpp:832-845): per vertex whether it touched its collision
 * plane in any substep (mHasContact), the contact point GetLocalContactPoint (in the body's local frame
 * before the step's recentring) and the contact normal GetContactNormal; plus the recentring offset of the
 * step. Off by default (it costs a byte per vertex per substep of stores). */
jsb_status jsb_set_contact_readback(jsb_context *ctx, int enable);
/* After a step with the readback on (synchronises the device): per vertex has_contact (0 / 1), contact point
 * and normal (3 floats each, zero without contact) and the colliding shape's index (the host-determined
 * table's order, or the order of the context colliders the body's bounds overlapped; -1 without contact),
 * and the recentring offset delta (local positions after the step = before - delta). Any output may be
 * NULL. */
jsb_status jsb_body_contacts(jsb_context *ctx, uint32_t body_id, uint8_t *has_contact, float *contact_points, float *normals,
                             int32_t *shape_index, float delta[3]);
/* ---- skinning (skinned constraints) --------------------------------------------------------- */
/* SoftBodyMotionProperties::SkinVertices (SoftBodyMotionProperties.cpp:1139-1230) for a body whose settings
 * have skinned constraints: the skinned positions from `num_joints` joint matrices (16 floats each, Mat44
 * columns, in the soft body's space) times the settings' inverse bind matrices and skin weights, their
 * normals from the skinned faces, the previous skinned positions kept for the interpolation over the next
 * step's iterations; hard_skin_all moves every skinned vertex to its skinned position and zeroes its
 * velocity. Call it between steps; the next step's ApplySkinConstraints (:509-571: back stop sphere and
 * maximum distance) use it. Synchronous (host arithmetic in the reference's operation order). Skinned bodies
 * run on the one-CTA and the thread-block-cluster paths (not in differentiable runs, not through
 * jsb_step_body_noalloc). */
jsb_status jsb_body_skin_vertices(jsb_context *ctx, uint32_t body_id, const float *joint_matrices, uint32_t num_joints,
                                  int hard_skin_all);
/* SetEnableSkinConstraints / SetSkinnedMaxDistanceMultiplier (SoftBodyMotionProperties.h:93-98). */
jsb_status jsb_body_set_skin_settings(jsb_context *ctx, uint32_t body_id, int enable_skin_constraints,
                                      float max_distance_multiplier);

/* After a step (synchronises the device): bit k of *mask is set when shape k of the body's host-determined
 * shapes is a sensor shape (JSB_MOTION_SENSOR) that a vertex with inverse mass > 0 penetrated at the start
 * of the step (DetermineSensorCollisions, SoftBodyMotionProperties.cpp:267-289: CollidingSensor::mHasContact;
 * the sensors of SoftBodyManifold::GetSensorContactBodyID are those with a set bit in any of their shapes).
 * 0 for a body without host-determined shapes. */
jsb_status jsb_body_sensor_contacts(jsb_context *ctx, uint32_t body_id, uint32_t *mask);

/* ---- stepping ----------------------------------------------------------------------------- */
/* PhysicsSystem::Update's soft-body part for every body in the context: InitializeUpdateContext,
 * DetermineCollidingShapes, DetermineCollisionPlanes, num_iterations x (pressure, integrate,
 * update groups, collision + velocity), UpdateSoftBodyState, body position += delta.
 * Batched form: all bodies advance in persistent launches fed from a work queue. */
jsb_status jsb_step(jsb_context *ctx, float dt, int collision_steps, jsb_stream stream);

/* Same step, one body per launch (the plain form; what CustomUpdate would map to). */
jsb_status jsb_step_plain(jsb_context *ctx, float dt, int collision_steps, jsb_stream stream);

/* Capture `num_steps` batched steps into a CUDA graph and replay it `repeats` times. */
jsb_status jsb_step_graph(jsb_context *ctx, float dt, int collision_steps, int num_steps, int repeats,
                          jsb_stream stream);

/* Wait for the context's work and report device-side errors (JSB_ERR_NONFINITE, JSB_ERR_TIMEOUT). */
jsb_status jsb_synchronize(jsb_context *ctx);

/* ---- readback ----------------------------------------------------------------------------- */
/* Body position (world) and local vertex positions/velocities (3 floats each, any may be NULL). */
jsb_status jsb_body_read(jsb_context *ctx, uint32_t body_id, float position[3], float *local_positions,
                         float *velocities);

/* SoftBodyMotionProperties::SaveState bytes for RestoreState; *len receives the size (call with
 * state == NULL to query). */
jsb_status jsb_body_save_state(jsb_context *ctx, uint32_t body_id, void *state, size_t capacity, size_t *len);
/* The body's local bounds and local predicted bounds after the last step ({min xyz, max xyz} each;
 * SoftBodyMotionProperties::mLocalBounds / mLocalPredictedBounds), which DetermineCollidingShapes grows by
 * the vertex radius for its broad-phase query (SoftBodyMotionProperties.cpp:229-236). */
jsb_status jsb_body_bounds(jsb_context *ctx, uint32_t body_id, float local_bounds[6], float predicted_bounds[6]);

/* Bulk transfer of all bodies' local positions and velocities in body order (used for the
 * host-buffer round trip): 3 floats per vertex each. */
jsb_status jsb_state_upload_all(jsb_context *ctx, const float *local_positions, const float *velocities,
                                jsb_stream stream);
jsb_status jsb_state_download_all(jsb_context *ctx, float *local_positions, float *velocities, jsb_stream stream);
/* World positions of every body (3 floats per body, body order; synchronous). World vertex positions
 * are body position + local position. */
jsb_status jsb_body_positions_all(jsb_context *ctx, float *positions);
jsb_status jsb_total_vertices(jsb_context *ctx, uint64_t *total);

/* ---- scheduling and autotuning ------------------------------------------------------------ */
/* Number of dependency levels of a body's constraint schedule per substep and total constraints. */
jsb_status jsb_body_schedule_info(jsb_context *ctx, uint32_t body_id, uint32_t *num_levels, uint32_t *num_constraints);

/* Host only (no device needed): the dependency-level schedule built for these settings bytes.
 * levels receives 4 x (num_levels + 2) uint32 {first record, end of bends, end of volumes, end of
 * edges}, records 4 x num_records uint32 (16-byte records), source num_records uint32
 * (type << 28 | index in the settings' constraint array; type 0 bend, 1 volume, 2 edge, 3 LRA).
 * Pass NULL arrays to query the sizes. */
jsb_status jsb_settings_schedule(const void *blob, size_t len, uint32_t *num_levels, uint32_t *num_records,
                                 uint32_t *levels, uint32_t *records, uint32_t *source);

/* Host only, opt-in and NOT the reference's order: regrouped settings bytes. Each constraint type is
 * reordered by a greedy colouring in the reference's sequence order (first fit over constraints of the
 * type sharing a written vertex; tethers also over their anchors) and every constraint goes into one
 * update group, which SoftBodyMotionProperties processes sequentially (volumes, bends, edges, LRA,
 * ProcessGroup :1030-1055), each type by colour. The bytes are a valid SaveBinaryState of
 * SoftBodySharedSettings (Jolt itself runs them the same way); their dependency schedule has about the
 * colour counts of the types added up as levels per substep (tens for a cloth, instead of the hundreds
 * to thousands of the reference's order), at the price of a different Gauss-Seidel order: results differ
 * from the reference's by what reordering the constraint sweep does. This replaces the reference's
 * SoftBodySharedSettings::Optimize grouping (SoftBodySharedSettings.cpp:613-1182) for callers who accept that.
 * Pass out = NULL to query *out_len. remap (may be NULL; num_edges + num_bends + num_volumes + num_lra
 * entries): for the edges, bends, volumes and LRA constraints in their new order, each one's index in the
 * input. Skinned constraints and rods are refused (JSB_ERR_UNSUPPORTED). */
jsb_status jsb_settings_regroup(const void *blob, size_t len, void *out, size_t capacity, size_t *out_len, uint32_t *remap);

/* Host only: the whole-step schedule (see jsb_set_step_walk) of these settings for `num_iterations`
 * substeps, in the padded device layout. levels receives 4 x num_levels uint32 {first slot, bend end |
 * volume end << 16, edge end | LRA end << 16, slots of the level} (ends relative to the first slot;
 * vertex slots from the LRA end on), records 4 x num_slots uint32 (padding slots have 0xffffffff in
 * their first word; a vertex slot is {vertex index, substep it enters, 0, 0}), source 2 x num_slots uint32 {type << 28 |
 * index, substep} (type 0 bend, 1 volume, 2 edge, 3 LRA, 4 vertex; 0xffffffff for padding). Sizes are
 * 0 when the settings have no whole-step schedule (num_iterations < 2, or a level of 65,536 slots or
 * more). Pass NULL arrays to query the sizes. */
jsb_status jsb_settings_step_schedule(const void *blob, size_t len, uint32_t num_iterations, uint32_t *num_levels,
                                      uint32_t *num_slots, uint32_t *levels, uint32_t *records, uint32_t *source);
/* Launch shape of the size bucket of bodies with vertex count <= max_vertices (and above the next
 * smaller bucket): threads per CTA in {32, 64, 128, 256, 512}; state_mode 0 keeps positions, velocities and
 * previous positions in shared memory when they fit, 1 keeps only positions there, 2 sends the
 * bucket's bodies to the thread-block-cluster path. The autotuner writes this table; the calls below
 * set or read it directly. Bodies whose positions do not fit one CTA's shared memory always take the
 * cluster path. */
jsb_status jsb_set_bucket_config(jsb_context *ctx, uint32_t max_vertices, uint32_t threads, uint32_t state_mode);
jsb_status jsb_set_bucket_threads(jsb_context *ctx, uint32_t max_vertices, uint32_t threads);
/* Thread-block-cluster path (bodies too large for one SM, up to 65,536 vertices; no counterpart in the
 * reference, whose SoftBodyMotionProperties::ParallelUpdate spreads one body over job-system threads,
 * SoftBodyMotionProperties.cpp:1057-1115): CTAs per cluster in {2, 4, 8, 16} (0 = the largest that fits)
 * and threads per CTA in {128, 256, 512}. The getter reports the shape in use after the launch groups
 * are built, and how many bodies take the path. */
jsb_status jsb_set_cluster_config(jsb_context *ctx, uint32_t cluster_size, uint32_t threads);
/* Whole-step walk (no counterpart in the reference; on by default): a body without pressure on the
 * one-CTA path walks one dependency-level schedule for its whole step, in which each vertex takes the
 * velocity update of the substep it leaves and the integration of the next one right after its own last
 * constraint (ApplyCollisionConstraintsAndUpdateVelocities and IntegratePositions are per-vertex passes,
 * SoftBodyMotionProperties.cpp:325-365, 700-825), so substeps overlap. Results are bitwise those of the
 * per-substep walk (enable = 0), which pressurised bodies and the cluster path keep; differentiable runs
 * tape and reverse the whole-step walk. It cannot change during a differentiable run. */
jsb_status jsb_set_step_walk(jsb_context *ctx, int enable);
jsb_status jsb_get_cluster_config(jsb_context *ctx, uint32_t *cluster_size, uint32_t *threads, uint32_t *num_bodies);
jsb_status jsb_get_bucket_config(jsb_context *ctx, uint32_t index, uint32_t *max_vertices, uint32_t *threads,
                                 uint32_t *state_mode);
/* Tunes the bucket table on the context's own bodies: a few uniform starting tables, then up to two
 * rounds of coordinate descent over each occupied bucket's (threads, state placement), every candidate
 * timed as whole batched steps from the same state; the bodies' state is restored afterwards. */
jsb_status jsb_autotune(jsb_context *ctx, float dt, int trials);

/* Kernel launches issued by the most recent jsb_step / jsb_step_plain / jsb_step_graph call. */
jsb_status jsb_last_launch_count(jsb_context *ctx, uint32_t *launches);

/* Time (ms, CUDA events on the launching stream) of the dominant solver kernel launches issued by the
 * last jsb_step_graph call, averaged per step. */
jsb_status jsb_last_kernel_ms(jsb_context *ctx, float *ms_per_step);

/* ---- differentiable runs (hand-written adjoint) ----------------------------------------------- */
/* Per-constraint compliance of one body, in the settings' constraint order (mEdgeConstraints /
 * mVolumeConstraints after SoftBodySharedSettings::Optimize); either array may be NULL. The body's
 * settings must not be shared with another body. */
jsb_status jsb_body_set_compliance(jsb_context *ctx, uint32_t body_id, const float *edge_compliance, uint32_t num_edges,
                                   const float *volume_compliance, uint32_t num_volumes);

/* A differentiable run of num_steps batched steps (dt, one collision step) of every body in the
 * context, starting from the current state. jsb_adjoint_forward runs the steps (up to until_step, so
 * that positions of intermediate steps can be read between calls) and stores a checkpoint every
 * checkpoint_every steps; jsb_adjoint_seed adds d loss / d (world) vertex positions
 * of one body after a given step (1 .. num_steps); jsb_adjoint_backward recomputes each checkpoint
 * segment with a tape and reverses it (collision active set frozen) and leaves the context at the
 * forward run's final state; jsb_adjoint_gradients returns d loss / d initial positions and
 * velocities (3 floats per vertex), d loss / d the body's step force (3 floats, jsb_body_set_step_force)
 * and d loss / d each edge and volume compliance (settings order); any output may be NULL
 * (jsb_adjoint_bend_gradients: d loss / d each dihedral bend's compliance). Dihedral bends are
 * differentiated through their signed angle: C = ACosApproximate-based angle - initial angle is smooth
 * in the angle, so the derivative stays bounded at flat triangle pairs, where ACosApproximate's own
 * derivative is not (it is the limit of the derivative there). Positions and the body position are related by the body's
 * recentering, which leaves world positions unchanged; the adjoint is taken in world coordinates. */
jsb_status jsb_adjoint_begin(jsb_context *ctx, float dt, int num_steps, int checkpoint_every);
jsb_status jsb_adjoint_forward(jsb_context *ctx, int until_step); /* -1 = all num_steps; may be called in pieces */
jsb_status jsb_adjoint_seed(jsb_context *ctx, int step, uint32_t body_id, const float *dl_dx);
jsb_status jsb_adjoint_backward(jsb_context *ctx);
/* Every body at once, in context vertex order (bodies in creation order, 3 floats per vertex):
 * seeds d loss / d world positions after `step`, and reads d loss / d initial positions, initial
 * velocities and per-body force (3 floats per body); NULL outputs are skipped. */
jsb_status jsb_adjoint_seed_all(jsb_context *ctx, int step, const float *dl_dx);
jsb_status jsb_adjoint_gradients_all(jsb_context *ctx, float *dl_dx0, float *dl_dv0, float *dl_dforce);
jsb_status jsb_adjoint_gradients(jsb_context *ctx, uint32_t body_id, float *dl_dx0, float *dl_dv0, float *dl_dforce,
                                 float *dl_dedge_compliance, float *dl_dvolume_compliance);
jsb_status jsb_adjoint_bend_gradients(jsb_context *ctx, uint32_t body_id, float *dl_dbend_compliance);
/* Device time (CUDA events) of the last differentiable run's phases, ms: the forward steps
 * (jsb_adjoint_forward, the last segment taped), the taped recomputation of the other segments and the
 * reverse steps (jsb_adjoint_backward). */
jsb_status jsb_adjoint_timings(jsb_context *ctx, float out_ms[3]);
/* Ends the run. Its device buffers (tape, checkpoints, adjoints) stay with the context and are reused,
 * grown when needed, by its next differentiable run; jsb_context_destroy frees them. */
jsb_status jsb_adjoint_end(jsb_context *ctx);

/* ---- allocation-free single-body step -------------------------------------------------------- */
/* Body record in device memory for jsb_step_body_noalloc: the body's world position, its local bounds
 * and predicted bounds (SoftBodyMotionProperties mLocalBounds / mLocalPredictedBounds, which the next
 * step's collider query uses), and the linear / angular velocity the step writes. */
typedef struct jsb_body_state {
    float position[3];
    float bounds_min[3], bounds_max[3];
    float predicted_min[3], predicted_max[3];
    float linear_velocity[3], angular_velocity[3];
} jsb_body_state;

/* Limits of jsb_step_body_noalloc: its scratch is a fixed array in the library's device memory. */
#define JSB_NOALLOC_MAX_VERTICES 16384
#define JSB_NOALLOC_MAX_SLOTS 65536   /* constraint slots of the padded schedule (constraints + padding) */
#define JSB_NOALLOC_MAX_LEVELS 8192   /* dependency levels per substep */
#define JSB_NOALLOC_MAX_FACES 16384
#define JSB_NOALLOC_MAX_COLLIDERS 16

/* One full step of ONE body without any device allocation (this entry point has no counterpart in
 * the reference; it is an addition for callers that cannot call cudaMalloc: engines that own all
 * device memory through their own fixed arenas or budgets, and frame loops that must not hit the
 * implicit synchronisation and latency spikes of a device allocation).
 *
 * The caller passes the settings bytes (SoftBodySharedSettings::SaveBinaryState) and creation
 * settings on the host, and the body's state in its own device memory: x_device = float4[N]
 * (local position, inverse mass in w), v_device = float4[N] (velocity, w ignored), state_device, and
 * error_device (device-side error bits OR-ed in: 1 = a non-finite position or velocity
 * (JSB_ERR_NONFINITE), 2 = more colliders overlap the body than are kept per step, 4 = the bounded wait
 * for the copies that stage the body's state gave up (JSB_ERR_TIMEOUT; the body is then left unchanged
 * and the call's results are not valid); clear it before the call). Colliders, gravity and force are
 * host values.
 *
 * Scratch (the constraint schedule, per-vertex previous positions, collision planes and shape indices)
 * lives in one static device array of about 2.4 MB that every GPU loading the library holds until
 * exit; sizes beyond the JSB_NOALLOC_* limits are rejected with JSB_ERR_CAPACITY. The first call on a
 * device resolves the array's device address (cudaGetSymbolAddress) and sets the kernel's shared
 * memory limit; make that first call before any stream capture. Every call shares the array and
 * leaves its contents behind (nothing in it needs to start at zero: each call overwrites what it
 * reads); calls whose work overlaps on the GPU (several streams, or host threads) race on it, so
 * serialise them.
 *
 * Host cost per call: the settings bytes are parsed and the body's dependency-level schedule is rebuilt
 * on the host every call (about 0.3 ms for a 900-vertex cloth on an x86 core), then copied into the
 * array from pageable host memory, so the call returns only once those copies have been staged. */
jsb_status jsb_step_body_noalloc(const void *settings_blob, size_t len, const jsb_creation_settings *creation,
                                 const jsb_collider *colliders, uint32_t num_colliders, const float gravity[3],
                                 const float force[3], float dt, void *x_device, void *v_device,
                                 jsb_body_state *state_device, uint32_t *error_device, jsb_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* JSB_H */
