// Settings parsing and the dependency-level schedule.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../kernels/device_types.h"

namespace jsb {

// Parsed SoftBodySharedSettings::SaveBinaryState bytes (SoftBodySharedSettings.cpp:1203-1236).
struct ParsedSettings {
    struct Vertex {
        float pos[3], vel[3], inv_mass;
    };
    struct Face {
        uint32_t v[3], material;
    };
    struct Edge {
        uint32_t v[2];
        float rest, compliance;
    };
    struct Bend {
        uint32_t v[4];
        float compliance, initial_angle;
    };
    struct Volume {
        uint32_t v[4];
        float six_rest_volume, compliance;
    };
    struct LRA {
        uint32_t v[2];
        float max_distance;
    };
    struct Group {
        uint32_t edge, lra, rod_ss, rod_bt, bend, volume, skinned;
    };
    struct Skinned {  // SoftBodySharedSettings::Skinned
        uint32_t vertex;
        struct {
            uint32_t inv_bind;
            float weight;
        } w[4];
        float max_distance, backstop_distance, backstop_radius;
        uint32_t normal_info;  // start in skinned_normals (low 24 bits), face count (high 8 bits)
    };
    struct InvBind {  // SoftBodySharedSettings::InvBind
        uint32_t joint;
        float m[16];  // Mat44 columns
    };
    std::vector<Vertex> vertices;
    std::vector<Face> faces;
    std::vector<Edge> edges;
    std::vector<Bend> bends;
    std::vector<Volume> volumes;
    std::vector<LRA> lras;
    std::vector<Group> groups;
    std::vector<Skinned> skinned;
    std::vector<uint32_t> skinned_normals;  // face indices
    std::vector<InvBind> inv_binds;
    uint32_t num_skinned = 0, num_rod_stretch_shear = 0, num_rod_bend_twist = 0, num_inv_bind = 0;
};

// Returns an empty string on success, else a description of the problem. `unsupported` is set when
// the bytes are well formed but use constraint types the GPU path does not implement.
std::string parse_settings(const void *blob, size_t len, ParsedSettings &out, bool &unsupported);

// Constraint type order inside one dependency level (matches the level descriptor fields).
enum RecordType : uint32_t { kBend = 0, kVolume = 1, kEdge = 2, kLRA = 3 };
// Skinned constraints (ApplySkinConstraints, one vertex each) share the edge slots of a level: their
// record is {vertex | substep << 16, kSkinRecord | skinned index, 0, 0} (an edge's second word is 0), the
// substep being set in whole-step schedules only. In `source` they have type 5.
constexpr uint32_t kSkinRecord = 0x80000000u;
constexpr uint32_t kSkinSource = 5;

struct Schedule {
    // levels[l] = {first record, end of bends, end of volumes, end of edges}; levels has
    // num_levels + 2 entries, the last two being sentinels {n, n, n, n}.
    std::vector<uint32_t> levels;  // 4 per entry
    std::vector<uint32_t> records;  // 4 per record
    std::vector<uint32_t> source;  // per record: type << 28 | index in the settings' array
    uint32_t num_levels = 0;
    uint32_t num_records = 0;
    uint32_t max_level_width = 0;

    // Device layout: the same records with every type group of a level padded to a multiple of 32
    // slots (padding slots hold kPadRecord), so a warp projects one constraint type and slot s of a
    // level is simply record start + s.
    //   padded_levels[l] = {first slot, end of bend slots, end of volume slots, end of edge slots}
    //   (ends relative to the first slot); num_levels + 2 entries with two sentinels.
    std::vector<uint32_t> padded_levels;
    std::vector<uint32_t> padded_records;  // 4 per slot
    std::vector<uint32_t> padded_source;   // per slot: source of the record, 0xffffffff for padding
    uint32_t num_slots = 0;
    uint32_t max_level_slots = 0;
};

constexpr uint32_t kPadRecord = 0xffffffffu;  // first word of a padding slot

// Builds the dependency-level schedule of one substep's constraint projection.
//
// Sequence: the update groups in order (parallel groups first, the non-parallel group last), and in
// each group volumes, dihedral bends, skinned constraints, edges, LRA (ProcessGroup,
// SoftBodyMotionProperties.cpp:1030-1055).
// Level of a constraint = 1 + the latest level that wrote one of its vertices, and for vertices it
// writes also 1 + the latest level that read them (LRA constraints only read their anchor vertex).
// Constraints of one level therefore touch disjoint written vertices, so any execution order inside a
// level reproduces the sequential result bit for bit.
Schedule build_schedule(const ParsedSettings &s);

// Dependency-level schedule of a whole step of `num_iterations` substeps (bodies without pressure).
//
// Between the constraint projections of substep k - 1 and k the reference runs two per-vertex passes:
// ApplyCollisionConstraintsAndUpdateVelocities (static colliders, SoftBodyMotionProperties.cpp:700-825)
// and IntegratePositions (:325-365). Each reads and writes only its own vertex, so a vertex can take
// both as soon as its own last constraint of substep k - 1 has been projected, and the next substep's
// constraints on it can follow, while other vertices are still in substep k - 1. The schedule walks the
// reference's whole sequence (substep 0 constraints, then per vertex "velocity update + integrate",
// then substep 1 constraints, ...) with the same level rule as build_schedule, the per-vertex pair
// being a fifth slot type on one vertex. Substep 0's integration and the last substep's velocity update
// stay bulk passes around the walk. Only pressure couples all vertices between substeps (the volume is
// a sum over every face), so pressurised bodies keep the per-substep walk.
//   levels[l] = {first slot, bend end | volume end << 16, edge end | LRA end << 16, slots of the level}
//   (ends relative to the first slot, each type padded to a multiple of 32 slots; vertex slots run from
//   the LRA end to the level's slot count; a vertex slot's record is {vertex index, substep entered, 0, 0}).
struct StepSchedule {
    std::vector<uint32_t> levels;   // 4 per level
    std::vector<uint32_t> records;  // 4 per slot
    std::vector<uint32_t> source;   // 2 per slot when asked for: {type << 28 | index, substep}; padding 0xffffffff
    uint32_t num_levels = 0;
    uint32_t num_slots = 0;
    uint32_t max_level_slots = 0;
    uint32_t num_iterations = 0;
};
enum : uint32_t { kVertexOp = 4 };

// Returns false (and leaves `out` empty) when a level holds 65,536 slots or more, or num_iterations < 2.
// `with_source` also fills `source` (for tests of the order).
bool build_step_schedule(const ParsedSettings &s, uint32_t num_iterations, StepSchedule &out, bool with_source = false);

// Opt-in regrouping (not the reference's constraint order). Reorders each constraint type by a greedy
// graph colouring in the reference's sequence order (first fit: a constraint takes the smallest colour
// no constraint of its type sharing a written vertex has; an LRA tether also avoids colours in which its
// anchor is written or its vertex is read), stably by colour, and puts every constraint into one update
// group, which the reference processes sequentially: volumes, bends, edges, LRA, each by colour. The
// bytes are valid SoftBodySharedSettings (SaveBinaryState layout, one group, no skinned constraints or
// rods), so the reference, the oracle and the GPU all run the new order the same way; the dependency
// levels of that order are about the colours of each type added up (tens per substep for a cloth, where
// the reference's order has hundreds or thousands). The result differs from the reference's order the
// way any other Gauss-Seidel order does. remap (edges, bends, volumes, LRA in their new order): the
// original index of each constraint within its type.
std::vector<uint8_t> regroup_settings(const ParsedSettings &s, std::vector<uint32_t> &remap);

// Staging chunks of a level schedule. The walkers stage a schedule's records and level descriptors
// into shared memory chunk by chunk, with one bulk copy of each per chunk, into the two halves of a
// ring (chunk c into half c % 2, two chunks in flight). A chunk is a run of consecutive levels whose
// slots fit `half_slots` and whose descriptors fit kStageLevels, or one wider level, of which the
// first half_slots slots are staged (the walker reads the rest in place).
//   chunk = {first level, end level, first slot, staged slots}, 4 uint32 each.
// levels4: per-substep layout (Schedule::padded_levels: a level's slots end where the next level's
// begin; num_levels + 2 entries) when per_substep, else the whole-step layout (StepSchedule::levels,
// slot count in the fourth word).
std::vector<uint32_t> build_stage_chunks(const std::vector<uint32_t> &levels4, uint32_t num_levels, bool per_substep,
                                         uint32_t half_slots);

}  // namespace jsb
