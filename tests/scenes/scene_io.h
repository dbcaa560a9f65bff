// Serialised scene ("JSBS"): the hand-off format between scene construction (this library's
// settings mirror, or Jolt itself in the reference driver) and whoever steps it (the C ABI, the CPU
// oracle, the tests).
//
//   char[4] 'JSBS'; u32 version = 1; u32 num_bodies; u32 num_colliders;
//   f32 gravity[3]; f32 dt; i32 collision_steps; i32 num_steps;
//   num_colliders x { i32 type; f32 position[3]; f32 half_extent[3]; f32 radius; f32 friction; f32 restitution }
//   num_bodies x { f32 position[3]; jsb_creation_settings (36 bytes); f32 force[3];
//                  u32 blob_len; blob_len bytes of SoftBodySharedSettings::SaveBinaryState }
#pragma once

#include <cstring>
#include <functional>
#include <string>

#include "scene_spec.h"

namespace jsb {
namespace scene {

template <class T>
inline void io_put(std::string &out, const T &v) {
    out.append(reinterpret_cast<const char *>(&v), sizeof(T));
}

// blob_of(mesh) returns the SaveBinaryState bytes for one body.
inline std::string serialize_scene(const SceneSpec &s, const std::function<std::string(const MeshSpec &)> &blob_of) {
    std::string out("JSBS", 4);
    io_put(out, uint32_t(1));
    io_put(out, uint32_t(s.bodies.size()));
    io_put(out, uint32_t(s.colliders.size()));
    for (int k = 0; k < 3; ++k) io_put(out, s.gravity[k]);
    io_put(out, s.dt);
    io_put(out, int32_t(s.collision_steps));
    io_put(out, int32_t(s.num_steps));
    for (const ColliderSpec &c : s.colliders) {
        io_put(out, int32_t(c.type));
        for (int k = 0; k < 3; ++k) io_put(out, c.position[k]);
        for (int k = 0; k < 3; ++k) io_put(out, c.half_extent[k]);
        io_put(out, c.radius);
        io_put(out, c.friction);
        io_put(out, c.restitution);
    }
    for (const BodySpec &b : s.bodies) {
        for (int k = 0; k < 3; ++k) io_put(out, b.position[k]);
        const CreationScalars &c = b.creation;
        io_put(out, c.num_iterations);
        io_put(out, c.linear_damping);
        io_put(out, c.max_linear_velocity);
        io_put(out, c.restitution);
        io_put(out, c.friction);
        io_put(out, c.pressure);
        io_put(out, c.gravity_factor);
        io_put(out, c.vertex_radius);
        io_put(out, uint8_t(c.update_position));
        io_put(out, uint8_t(c.make_rotation_identity));
        io_put(out, uint8_t(c.allow_sleeping));
        io_put(out, uint8_t(c.faces_double_sided));
        for (int k = 0; k < 3; ++k) io_put(out, b.force[k]);
        std::string blob = blob_of(b.mesh);
        io_put(out, uint32_t(blob.size()));
        out += blob;
    }
    return out;
}

// Parses "k=v k=v" parameter strings.
inline bool param_get(const std::string &params, const char *key, long &value) {
    std::string k = std::string(key) + "=";
    size_t pos = 0;
    while (pos < params.size()) {
        while (pos < params.size() && params[pos] == ' ') ++pos;
        size_t end = params.find(' ', pos);
        if (end == std::string::npos) end = params.size();
        if (params.compare(pos, k.size(), k) == 0) {
            value = std::stol(params.substr(pos + k.size(), end - pos - k.size()));
            return true;
        }
        pos = end;
    }
    return false;
}

// Builds a named workload with optional overrides; returns false for an unknown name.
inline bool make_named_scene(const std::string &name, const std::string &params, SceneSpec &out) {
    auto geti = [&](const char *k, long d) {
        long v;
        return param_get(params, k, v) ? v : d;
    };
    if (name == "pinned_cloth")
        out = make_pinned_cloth(uint32_t(geti("n", 30)), int(geti("steps", 300)));
    else if (name == "uneven_batch")
        out = make_uneven_batch(uint64_t(geti("seed", 2)), uint32_t(geti("n_cloth", 384)), uint32_t(geti("n_cube", 128)),
                                int(geti("steps", 240)), uint32_t(geti("cloth_min", 8)), uint32_t(geti("cloth_max", 64)),
                                uint32_t(geti("cube_min", 4)), uint32_t(geti("cube_max", 12)));
    else if (name == "large_cloth")
        out = make_large_cloth(uint32_t(geti("n", 256)), int(geti("steps", 600)), geti("bends", 1) != 0);
    else if (name == "diff_cloth")
        out = make_diff_cloth(uint64_t(geti("seed", 4)), uint32_t(geti("n", 64)), int(geti("steps", 120)), geti("bends", 0) != 0,
                              float(geti("wave_mm", 0)) * 1.0e-3f);
    else if (name == "diff_batch")
        out = make_diff_batch(uint64_t(geti("seed", 5)), uint32_t(geti("n_cloth", 192)), uint32_t(geti("n_cube", 64)),
                              int(geti("steps", 90)), float(geti("drop_mm", 1000)) * 0.001f);
    else if (name == "coupling")
        out = make_coupling(int(geti("steps", 90)), geti("hulls", 0) != 0, geti("sensors", 0) != 0);
    else if (name == "skinned_cloth")
        out = make_skinned_cloth(int(geti("steps", 90)));
    else if (name == "shapes_drop")
        out = make_shapes_drop(uint64_t(geti("seed", 7)), int(geti("steps", 150)));
    else
        return false;
    long it;
    if (param_get(params, "iterations", it))
        for (auto &b : out.bodies) b.creation.num_iterations = uint32_t(it);
    long sleep;
    if (param_get(params, "sleep", sleep))  // SoftBodyCreationSettings::mAllowSleeping of every body
        for (auto &b : out.bodies) b.creation.allow_sleeping = sleep != 0;
    return true;
}

}  // namespace scene
}  // namespace jsb
