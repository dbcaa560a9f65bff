// Seeded synthetic soft-body scenes used by the tests, the benchmark and the reference driver.
//
// A scene is described with plain data (vertex positions, inverse masses, faces, explicit
// edges/tetrahedra, per-vertex constraint attributes, creation scalars, colliders). The same
// description is turned into SoftBodySharedSettings either by Jolt's own API
// (oracle/ref_driver.cpp, where the reference is available) or by this project's host mirror
// (shared_settings.cpp), so both sides simulate byte-identical inputs.
//
// Cloth layout follows Samples/Utils/SoftBodyCreator.cpp:11-56 (grid in the XZ plane, centred on
// the origin, two triangles per cell, CreateConstraints + Optimize). Tetrahedral cubes use a
// 5-tetrahedra-per-cell decomposition with alternating cell parity (Jolt's sCreateCube,
// Jolt/Physics/SoftBody/SoftBodySharedSettings.cpp:1333-1484, uses 6 per cell; the 5-tet variant is
// this project's own generator) with explicit edges, volumes and outward surface faces.
//
// All random draws come from std::mt19937_64 (fully specified by the C++ standard) through the
// distributions below, which are written out here so results do not depend on the standard
// library's implementation-defined distributions.
#pragma once

#include <cmath>
#include <cstdint>
#include <random>
#include <vector>
#include <array>
#include <algorithm>

namespace jsb {
namespace scene {

// ---------------------------------------------------------------------------------------------
// Random numbers
// ---------------------------------------------------------------------------------------------
class Rng {
public:
    explicit Rng(uint64_t seed) : eng_(seed) {}
    // Uniform double in [0, 1) from the top 53 bits.
    double uniform() { return double(eng_() >> 11) * (1.0 / 9007199254740992.0); }
    // Uniform integer in [lo, hi] (inclusive).
    int64_t uniform_int(int64_t lo, int64_t hi) {
        uint64_t span = uint64_t(hi - lo) + 1;
        return lo + int64_t(uint64_t(uniform() * double(span)) % span);
    }
    // Log-uniform in [lo, hi].
    double log_uniform(double lo, double hi) {
        double a = std::log(lo), b = std::log(hi);
        return std::exp(a + (b - a) * uniform());
    }
    // Standard normal (Box-Muller, one draw per call).
    double normal() {
        double u1 = uniform();
        double u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }

private:
    std::mt19937_64 eng_;
};

// ---------------------------------------------------------------------------------------------
// Plain scene description
// ---------------------------------------------------------------------------------------------
enum class BendType : int { None = 0, Distance = 1, Dihedral = 2 };
enum class LRAType : int { None = 0, EuclideanDistance = 1, GeodesicDistance = 2 };

struct VertexAttributes {  // mirrors SoftBodySharedSettings::VertexAttributes (SoftBodySharedSettings.h:38-50)
    float compliance = 0.0f;
    float shear_compliance = 0.0f;
    float bend_compliance = 3.402823466e+38f;
    LRAType lra_type = LRAType::None;
    float lra_max_distance_multiplier = 1.0f;
};

struct MeshSpec {
    std::vector<std::array<float, 3>> positions;
    std::vector<std::array<float, 3>> velocities;  // initial velocity per vertex
    std::vector<float> inv_mass;
    std::vector<std::array<uint32_t, 3>> faces;
    // Either constraints come from CreateConstraints(attributes, bend_type) ...
    bool create_constraints = true;
    VertexAttributes attributes;
    BendType bend_type = BendType::Dihedral;
    // ... or they are explicit (edges + tetrahedra), followed by CalculateEdgeLengths and
    // CalculateVolumeConstraintVolumes.
    std::vector<std::array<uint32_t, 2>> edges;
    std::vector<float> edge_compliance;  // per explicit edge
    std::vector<std::array<uint32_t, 4>> volumes;
    std::vector<float> volume_compliance;  // per tetrahedron
    // Optional per-edge compliance written after Optimize, indexed in the optimized edge order.
    std::vector<float> post_optimize_edge_compliance;
    // Skinned constraints (reference driver only): per constraint the vertex, up to 4 (inverse bind index,
    // weight) pairs, max distance, back stop distance and radius; inverse bind matrices (joint, Mat44
    // columns). Added before Optimize, with CalculateSkinnedConstraintNormals.
    struct Skin {
        uint32_t vertex;
        std::array<std::pair<uint32_t, float>, 4> weights;
        float max_distance, backstop_distance, backstop_radius;
    };
    std::vector<Skin> skinned;
    std::vector<std::pair<uint32_t, std::array<float, 16>>> inv_binds;
};

struct CreationScalars {  // mirrors SoftBodyCreationSettings (SoftBodyCreationSettings.h:61-72)
    uint32_t num_iterations = 5;
    float linear_damping = 0.1f;
    float max_linear_velocity = 500.0f;
    float restitution = 0.0f;
    float friction = 0.2f;
    float pressure = 0.0f;
    float gravity_factor = 1.0f;
    float vertex_radius = 0.0f;
    bool update_position = true;
    bool make_rotation_identity = true;
    bool allow_sleeping = false;
    bool faces_double_sided = false;
};

struct BodySpec {
    MeshSpec mesh;
    float position[3] = {0, 0, 0};
    CreationScalars creation;
    float force[3] = {0, 0, 0};  // added with AddForce before every step
};

enum class ColliderType : int { Box = 0, Sphere = 1, Capsule = 2, Cylinder = 3, Hull = 4 };

struct ColliderSpec {  // a static rigid body with one convex shape (capsules and cylinders along Y)
    ColliderType type = ColliderType::Box;
    float position[3] = {0, 0, 0};
    float half_extent[3] = {1, 1, 1};  // box; [1]: half height of a capsule's cylinder part / a cylinder
    float radius = 1.0f;               // sphere, capsule, cylinder
    float friction = 0.2f;
    float restitution = 0.0f;
};

// A rigid body that only the reference driver creates and simulates with Jolt's own rigid-body solver
// (scenes of two-way coupling); it is not part of the serialised scene: the soft bodies' colliding
// shapes, as the reference determined them each step, reach the GPU and the oracle through the
// host-determined colliding-shape tables.
struct RigidSpec {
    ColliderType type = ColliderType::Box;
    int motion = 2;                        // EMotionType: 0 static, 1 kinematic, 2 dynamic
    float position[3] = {0, 0, 0};
    float rotation[4] = {0, 0, 0, 1};      // quaternion x, y, z, w
    float half_extent[3] = {1, 1, 1};      // box; [1]: half height of a capsule's cylinder part / a cylinder
    float radius = 1.0f;
    float mass = 1.0f;                     // dynamic bodies (inertia from the shape)
    float friction = 0.2f;
    float restitution = 0.0f;
    float velocity[3] = {0, 0, 0};
    float angular_velocity[3] = {0, 0, 0};
    std::vector<std::array<float, 3>> hull_points;  // ColliderType::Hull: the points the hull is built from
    bool sensor = false;                   // BodyCreationSettings::mIsSensor
};

struct SceneSpec {
    std::vector<BodySpec> bodies;
    std::vector<ColliderSpec> colliders;
    std::vector<RigidSpec> rigid;  // reference driver only
    float gravity[3] = {0.0f, -9.81f, 0.0f};
    float dt = 1.0f / 60.0f;
    int collision_steps = 1;
    int num_steps = 1;
};

// ---------------------------------------------------------------------------------------------
// Builders
// ---------------------------------------------------------------------------------------------

// Cloth grid in the XZ plane like SoftBodyCreator::CreateCloth (SoftBodyCreator.cpp:11-56).
// pinned(x, z) returns true for kinematic vertices.
template <class Pinned>
inline MeshSpec make_cloth(uint32_t nx, uint32_t nz, float spacing, Pinned pinned) {
    MeshSpec m;
    const float off_x = -0.5f * spacing * float(nx - 1);
    const float off_z = -0.5f * spacing * float(nz - 1);
    for (uint32_t z = 0; z < nz; ++z)
        for (uint32_t x = 0; x < nx; ++x) {
            float px = off_x + float(x) * spacing;
            float pz = off_z + float(z) * spacing;
            m.positions.push_back({px, 0.0f, pz});
            m.velocities.push_back({0.0f, 0.0f, 0.0f});
            m.inv_mass.push_back(pinned(x, z) ? 0.0f : 1.0f);
        }
    auto vi = [nx](uint32_t x, uint32_t z) { return x + z * nx; };
    for (uint32_t z = 0; z + 1 < nz; ++z)
        for (uint32_t x = 0; x + 1 < nx; ++x) {
            m.faces.push_back({vi(x, z), vi(x, z + 1), vi(x + 1, z + 1)});
            m.faces.push_back({vi(x, z), vi(x + 1, z + 1), vi(x + 1, z)});
        }
    return m;
}

// Cube of n x n x n cells of size `cell`, 5 tetrahedra per cell with alternating parity so that
// neighbouring cells share face diagonals. Edges are all unique tetrahedron edges (in first-seen
// order), faces are the outward-oriented boundary triangles (diagonals matching the tets).
inline MeshSpec make_tet_cube(uint32_t n, float cell, float edge_compliance, float volume_compliance) {
    MeshSpec m;
    m.create_constraints = false;
    const uint32_t g = n + 1;
    const float off = -0.5f * cell * float(n);
    for (uint32_t z = 0; z < g; ++z)
        for (uint32_t y = 0; y < g; ++y)
            for (uint32_t x = 0; x < g; ++x) {
                m.positions.push_back({off + float(x) * cell, off + float(y) * cell, off + float(z) * cell});
                m.velocities.push_back({0.0f, 0.0f, 0.0f});
                m.inv_mass.push_back(1.0f);
            }
    auto vi = [g](uint32_t x, uint32_t y, uint32_t z) { return x + y * g + z * g * g; };
    // corner c = bits (x | y<<1 | z<<2)
    static const int even_tets[5][4] = {{0, 3, 5, 6}, {1, 0, 3, 5}, {2, 0, 6, 3}, {4, 0, 5, 6}, {7, 3, 6, 5}};
    static const int odd_tets[5][4] = {{1, 2, 4, 7}, {0, 1, 4, 2}, {3, 1, 2, 7}, {5, 1, 7, 4}, {6, 2, 4, 7}};
    std::vector<uint64_t> edge_keys;
    auto add_edge = [&](uint32_t a, uint32_t b) {
        uint32_t lo = std::min(a, b), hi = std::max(a, b);
        uint64_t key = (uint64_t(lo) << 32) | hi;
        for (uint64_t k : edge_keys)
            if (k == key) return;
        edge_keys.push_back(key);
    };
    std::vector<std::vector<uint64_t>> edge_buckets(g * g * g);  // faster duplicate check
    auto add_edge_fast = [&](uint32_t a, uint32_t b) {
        uint32_t lo = std::min(a, b), hi = std::max(a, b);
        for (uint64_t k : edge_buckets[lo])
            if (k == hi) return;
        edge_buckets[lo].push_back(hi);
        m.edges.push_back({lo, hi});
        m.edge_compliance.push_back(edge_compliance);
    };
    (void)add_edge;
    for (uint32_t z = 0; z < n; ++z)
        for (uint32_t y = 0; y < n; ++y)
            for (uint32_t x = 0; x < n; ++x) {
                uint32_t c[8];
                for (int b = 0; b < 8; ++b) c[b] = vi(x + (b & 1), y + ((b >> 1) & 1), z + ((b >> 2) & 1));
                const int(*tets)[4] = ((x + y + z) & 1) ? odd_tets : even_tets;
                for (int t = 0; t < 5; ++t) {
                    std::array<uint32_t, 4> tet = {c[tets[t][0]], c[tets[t][1]], c[tets[t][2]], c[tets[t][3]]};
                    // make the orientation positive: (x2-x1) x (x3-x1) . (x4-x1) > 0
                    auto P = [&](uint32_t i) { return m.positions[i]; };
                    double a[3], b2[3], d[3];
                    for (int k = 0; k < 3; ++k) {
                        a[k] = double(P(tet[1])[k]) - P(tet[0])[k];
                        b2[k] = double(P(tet[2])[k]) - P(tet[0])[k];
                        d[k] = double(P(tet[3])[k]) - P(tet[0])[k];
                    }
                    double det = (a[1] * b2[2] - a[2] * b2[1]) * d[0] + (a[2] * b2[0] - a[0] * b2[2]) * d[1] +
                                 (a[0] * b2[1] - a[1] * b2[0]) * d[2];
                    if (det < 0) std::swap(tet[2], tet[3]);
                    m.volumes.push_back(tet);
                    m.volume_compliance.push_back(volume_compliance);
                    for (int i = 0; i < 4; ++i)
                        for (int j = i + 1; j < 4; ++j) add_edge_fast(tet[i], tet[j]);
                }
            }
    // Boundary faces: each boundary quad is split along the diagonal that the adjacent cell's
    // tetrahedra use, i.e. the diagonal between the two corners of the cell's "even" class.
    // For a cell with parity p the central tetrahedron uses corners of class p ^ 0; a face of the
    // cell contains two corners of each class; the diagonal is the pair of class (parity of cell).
    auto emit_quad = [&](uint32_t a, uint32_t b, uint32_t c2, uint32_t d, bool diag_ac, const float normal[3]) {
        // a, b, c2, d go around the quad; diagonal a-c2 if diag_ac, else b-d
        std::array<uint32_t, 3> t1, t2;
        if (diag_ac) {
            t1 = {a, b, c2};
            t2 = {a, c2, d};
        } else {
            t1 = {a, b, d};
            t2 = {b, c2, d};
        }
        for (auto *t : {&t1, &t2}) {
            auto &tr = *t;
            double e1[3], e2[3];
            for (int k = 0; k < 3; ++k) {
                e1[k] = double(m.positions[tr[1]][k]) - m.positions[tr[0]][k];
                e2[k] = double(m.positions[tr[2]][k]) - m.positions[tr[0]][k];
            }
            double nrm[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            if (nrm[0] * normal[0] + nrm[1] * normal[1] + nrm[2] * normal[2] < 0) std::swap(tr[1], tr[2]);
            m.faces.push_back(tr);
        }
    };
    auto parity_even_corner = [](uint32_t cx, uint32_t cy, uint32_t cz, uint32_t vx, uint32_t vy, uint32_t vz) {
        // corner class relative to the cell: even if (bits sum) even; central tet of an even cell
        // uses the even corners, of an odd cell the odd corners; diagonals on faces connect
        // corners of the class used by the central tet.
        uint32_t bits = (vx - cx) + (vy - cy) + (vz - cz);
        uint32_t cell_par = (cx + cy + cz) & 1;
        return ((bits & 1) == cell_par);
    };
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j < n; ++j) {
            // faces x = 0 and x = n (cells (0, i, j) and (n - 1, i, j))
            for (int side = 0; side < 2; ++side) {
                uint32_t cx = side ? n - 1 : 0, vx = side ? n : 0;
                const float nrm[3] = {side ? 1.0f : -1.0f, 0, 0};
                uint32_t a = vi(vx, i, j), b = vi(vx, i + 1, j), c2 = vi(vx, i + 1, j + 1), d = vi(vx, i, j + 1);
                emit_quad(a, b, c2, d, parity_even_corner(cx, i, j, vx, i, j), nrm);
            }
            // faces y = 0 and y = n
            for (int side = 0; side < 2; ++side) {
                uint32_t cy = side ? n - 1 : 0, vy = side ? n : 0;
                const float nrm[3] = {0, side ? 1.0f : -1.0f, 0};
                uint32_t a = vi(i, vy, j), b = vi(i + 1, vy, j), c2 = vi(i + 1, vy, j + 1), d = vi(i, vy, j + 1);
                emit_quad(a, b, c2, d, parity_even_corner(i, cy, j, i, vy, j), nrm);
            }
            // faces z = 0 and z = n
            for (int side = 0; side < 2; ++side) {
                uint32_t cz = side ? n - 1 : 0, vz = side ? n : 0;
                const float nrm[3] = {0, 0, side ? 1.0f : -1.0f};
                uint32_t a = vi(i, j, vz), b = vi(i + 1, j, vz), c2 = vi(i + 1, j + 1, vz), d = vi(i, j + 1, vz);
                emit_quad(a, b, c2, d, parity_even_corner(i, j, cz, i, j, vz), nrm);
            }
        }
    return m;
}

// ---------------------------------------------------------------------------------------------
// The five workloads
// ---------------------------------------------------------------------------------------------

// Plain single cloth: 30x30 grid, 0.75 m spacing in the XZ plane at y = 10, inverse mass 1 with the
// two corners of the far row (z = 29) pinned, edge/shear compliance 1e-5, dihedral bend compliance
// 1e-4, 5 iterations, damping 0.1, no colliders, 300 steps of 1/60 s.
inline SceneSpec make_pinned_cloth(uint32_t n = 30, int steps = 300) {
    SceneSpec s;
    BodySpec b;
    b.mesh = make_cloth(n, n, 0.75f, [n](uint32_t x, uint32_t z) { return z == n - 1 && (x == 0 || x == n - 1); });
    b.mesh.attributes = VertexAttributes{1.0e-5f, 1.0e-5f, 1.0e-4f};
    b.mesh.bend_type = BendType::Dihedral;
    b.position[1] = 10.0f;
    s.bodies.push_back(b);
    s.num_steps = steps;
    return s;
}

// Layout helper: places `count` bodies on a square grid in XZ with the given pitch, centred on the
// origin, and returns the floor box that covers them (top face at y = 0).
inline void grid_place(SceneSpec &s, float pitch, float height_base) {
    size_t count = s.bodies.size();
    uint32_t side = 1;
    while (size_t(side) * side < count) ++side;
    float off = -0.5f * pitch * float(side - 1);
    for (size_t i = 0; i < count; ++i) {
        uint32_t gx = uint32_t(i % side), gz = uint32_t(i / side);
        s.bodies[i].position[0] = off + pitch * float(gx);
        s.bodies[i].position[2] = off + pitch * float(gz);
        s.bodies[i].position[1] += height_base;
    }
    ColliderSpec floor;
    floor.type = ColliderType::Box;
    float half = 0.5f * pitch * float(side) + pitch;
    floor.half_extent[0] = half;
    floor.half_extent[1] = 1.0f;
    floor.half_extent[2] = half;
    floor.position[0] = 0.0f;
    floor.position[1] = -1.0f;
    floor.position[2] = 0.0f;
    s.colliders.push_back(floor);
}

// Cloth with one randomly chosen border row/column pinned (0: z = 0, 1: z = n-1, 2: x = 0, 3: x = n-1).
inline MeshSpec make_edge_pinned_cloth(uint32_t n, float spacing, int side) {
    return make_cloth(n, n, spacing, [n, side](uint32_t x, uint32_t z) {
        switch (side) {
            case 0: return z == 0;
            case 1: return z == n - 1;
            case 2: return x == 0;
            default: return x == n - 1;
        }
    });
}

// Batch of uneven bodies: `n_cloth` cloths with side U{8..64} (spacing 0.1 m, dihedral bends with
// compliance 1e-4, edge/shear compliance log-U[1e-7, 1e-3], one border row pinned) and `n_cube`
// 5-tet cubes with U{4..12} cells of 1 m (volume compliance log-U[1e-8, 1e-5], edge compliance 0,
// pressure 0 or 1e3 with probability 1/2), on a seeded grid above a static box floor; 5 iterations,
// 240 steps of 1/60 s.
inline SceneSpec make_uneven_batch(uint64_t seed = 2, uint32_t n_cloth = 384, uint32_t n_cube = 128, int steps = 240,
                                   uint32_t cloth_min = 8, uint32_t cloth_max = 64, uint32_t cube_min = 4,
                                   uint32_t cube_max = 12) {
    SceneSpec s;
    Rng rng(seed);
    for (uint32_t i = 0; i < n_cloth; ++i) {
        BodySpec b;
        uint32_t n = uint32_t(rng.uniform_int(cloth_min, cloth_max));
        float c = float(rng.log_uniform(1e-7, 1e-3));
        int side = int(rng.uniform_int(0, 3));
        b.mesh = make_edge_pinned_cloth(n, 0.1f, side);
        b.mesh.attributes = VertexAttributes{c, c, 1.0e-4f};
        b.mesh.bend_type = BendType::Dihedral;
        b.position[1] = 0.5f * 0.1f * float(n) + 1.0f;
        s.bodies.push_back(b);
    }
    for (uint32_t i = 0; i < n_cube; ++i) {
        BodySpec b;
        uint32_t n = uint32_t(rng.uniform_int(cube_min, cube_max));
        float vc = float(rng.log_uniform(1e-8, 1e-5));
        bool pressure = rng.uniform() < 0.5;
        b.mesh = make_tet_cube(n, 1.0f, 0.0f, vc);
        b.creation.pressure = pressure ? 1.0e3f : 0.0f;
        b.position[1] = 0.5f * float(n) + 1.0f;
        s.bodies.push_back(b);
    }
    grid_place(s, 14.0f, 0.0f);
    s.num_steps = steps;
    return s;
}

// Single large cloth: n x n grid (default 256), 0.02 m spacing, 4 corners pinned, Euclidean LRA
// tethers, edge compliance 1e-6, bend compliance 1e-3, 8 iterations, dropped from y = 3 (1 m above
// the top of a static sphere of radius 1 centred at y = 1) onto the sphere resting on a box floor
// whose top is at y = 0; 600 steps of 1/60 s. bends = false leaves out the dihedral bends (a tethered
// cloth that differentiable runs accept).
inline SceneSpec make_large_cloth(uint32_t n = 256, int steps = 600, bool bends = true) {
    SceneSpec s;
    BodySpec b;
    b.mesh = make_cloth(n, n, 0.02f, [n](uint32_t x, uint32_t z) {
        return (x == 0 || x == n - 1) && (z == 0 || z == n - 1);
    });
    b.mesh.attributes = VertexAttributes{1.0e-6f, 1.0e-6f, bends ? 1.0e-3f : 3.402823466e+38f, LRAType::EuclideanDistance, 1.0f};
    b.mesh.bend_type = bends ? BendType::Dihedral : BendType::None;
    b.creation.num_iterations = 8;
    b.position[1] = 3.0f;
    s.bodies.push_back(b);
    ColliderSpec floor;
    floor.type = ColliderType::Box;
    floor.half_extent[0] = 20.0f;
    floor.half_extent[1] = 1.0f;
    floor.half_extent[2] = 20.0f;
    floor.position[1] = -1.0f;
    s.colliders.push_back(floor);
    ColliderSpec sphere;
    sphere.type = ColliderType::Sphere;
    sphere.radius = 1.0f;
    sphere.position[1] = 1.0f;
    s.colliders.push_back(sphere);
    s.num_steps = steps;
    return s;
}

// Differentiable single cloth: n x n (default 64), 0.05 m spacing, top row (z = n-1) pinned, edges
// only (bends = true adds dihedral bends of compliance 1e-4), per-edge compliance log-U[1e-6, 1e-4] assigned in optimized edge order, initial
// velocities N(0, 0.1) m/s per component; 120 steps.
// A 16 x 16 cloth (0.1 m spacing) hanging from two joints (reference driver only: the reference's
// SkinVertices is called before every step with the joints' matrices, which the driver records): the top
// row kinematic on joint 0 (max distance 0), the other rows skinned to joints 0 and 1 blended by row, with
// max distances growing down the cloth and a back stop sphere on every other row.
inline SceneSpec make_skinned_cloth(int steps = 90) {
    SceneSpec s;
    BodySpec b;
    const uint32_t n = 16;
    b.mesh = make_cloth(n, n, 0.1f, [](uint32_t, uint32_t) { return false; });
    b.mesh.attributes = VertexAttributes{1.0e-5f, 1.0e-5f, 1.0e-3f};
    b.mesh.bend_type = BendType::Dihedral;
    for (uint32_t z = 0; z < n; ++z)
        for (uint32_t x = 0; x < n; ++x) {
            MeshSpec::Skin k;
            k.vertex = x + z * n;
            const float t = float(z) / float(n - 1);
            k.weights = {{{0u, 1.0f - t}, {1u, t}, {0u, 0.0f}, {0u, 0.0f}}};
            if (z == 0) k.weights = {{{0u, 1.0f}, {0u, 0.0f}, {0u, 0.0f}, {0u, 0.0f}}};
            k.max_distance = z == 0 ? 0.0f : 0.02f + 0.01f * float(z);
            k.backstop_distance = (z & 1) ? 0.01f : k.max_distance;  // a back stop on odd rows only
            k.backstop_radius = 0.3f;
            b.mesh.skinned.push_back(k);
        }
    std::array<float, 16> ident{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::array<float, 16> down = ident;
    down[14] = -0.6f;  // joint 1 binds 0.6 m along the cloth (+z): its inverse bind matrix moves back by that
    b.mesh.inv_binds = {{0u, ident}, {1u, down}};
    b.position[1] = 1.5f;
    s.bodies.push_back(b);
    s.num_steps = steps;
    return s;
}

// wave: amplitude (m) of a height field y = wave sin(2 pi x / 0.8 m) sin(2 pi z / 0.8 m) laid over the
// grid, so that neighbouring triangles start folded by up to about 0.3 rad instead of flat.
inline SceneSpec make_diff_cloth(uint64_t seed = 4, uint32_t n = 64, int steps = 120, bool bends = false, float wave = 0.0f) {
    SceneSpec s;
    Rng rng(seed);
    BodySpec b;
    b.mesh = make_cloth(n, n, 0.05f, [n](uint32_t, uint32_t z) { return z == n - 1; });
    if (wave != 0.0f) {
        const double k = 2.0 * 3.14159265358979323846 / 0.8;
        for (auto &p : b.mesh.positions) p[1] = float(double(wave) * std::sin(k * double(p[0])) * std::sin(k * double(p[2])));
    }
    b.mesh.attributes = VertexAttributes{1.0e-5f, 1.0e-5f, bends ? 1.0e-4f : 3.402823466e+38f};
    b.mesh.bend_type = bends ? BendType::Dihedral : BendType::None;
    for (size_t v = 0; v < b.mesh.velocities.size(); ++v)
        for (int k = 0; k < 3; ++k) b.mesh.velocities[v][k] = float(0.1 * rng.normal());
    b.position[1] = 2.0f;
    // edge count is known only after CreateConstraints; draw enough values for any n x n grid
    size_t max_edges = size_t(4) * n * n;
    b.mesh.post_optimize_edge_compliance.resize(max_edges);
    for (auto &c : b.mesh.post_optimize_edge_compliance) c = float(rng.log_uniform(1e-6, 1e-4));
    s.bodies.push_back(b);
    s.num_steps = steps;
    return s;
}

// Differentiable batch: `n_cloth` cloths with side U{16..48} (0.05 m spacing, edges only, one border
// row pinned) and `n_cube` 5-tet cubes with U{4..8} cells of 0.25 m and pressure 5e2; per-body
// force N(0, 2 N) per axis, initial velocity N(0, 0.5 m/s); static box floor and a sphere of
// radius 0.5; 90 steps with 5 iterations. drop_height: gap between the bodies and the floor level.
inline SceneSpec make_diff_batch(uint64_t seed = 5, uint32_t n_cloth = 192, uint32_t n_cube = 64, int steps = 90,
                                 float drop_height = 1.0f) {
    SceneSpec s;
    Rng rng(seed);
    for (uint32_t i = 0; i < n_cloth + n_cube; ++i) {
        BodySpec b;
        if (i < n_cloth) {
            uint32_t n = uint32_t(rng.uniform_int(16, 48));
            int side = int(rng.uniform_int(0, 3));
            b.mesh = make_edge_pinned_cloth(n, 0.05f, side);
            b.mesh.attributes = VertexAttributes{1.0e-5f, 1.0e-5f, 3.402823466e+38f};
            b.mesh.bend_type = BendType::None;
            b.position[1] = 0.5f * 0.05f * float(n) + drop_height;
        } else {
            uint32_t n = uint32_t(rng.uniform_int(4, 8));
            b.mesh = make_tet_cube(n, 0.25f, 0.0f, 1.0e-6f);
            b.creation.pressure = 5.0e2f;
            b.position[1] = 0.5f * 0.25f * float(n) + drop_height;
        }
        for (int k = 0; k < 3; ++k) b.force[k] = float(2.0 * rng.normal());
        float v0[3];
        for (int k = 0; k < 3; ++k) v0[k] = float(0.5 * rng.normal());
        for (auto &v : b.mesh.velocities) v = {v0[0], v0[1], v0[2]};
        s.bodies.push_back(b);
    }
    grid_place(s, 4.0f, 0.0f);
    ColliderSpec sphere;
    sphere.type = ColliderType::Sphere;
    sphere.radius = 0.5f;
    sphere.position[1] = 0.5f;
    s.colliders.push_back(sphere);
    s.num_steps = steps;
    return s;
}

// Bodies dropped onto every static shape type: a box floor (top at y = 0) and, standing on it, a
// capsule (radius 0.4, cylinder half height 0.5), a cylinder (radius 0.5, half height 0.4), a flat
// cylinder (radius 0.8, half height 0.1) and a sphere (radius 0.5), 3 m apart along X. Over each shape a
// 16 x 16 cloth (0.08 m spacing, dihedral bends, unpinned) and a 4-cell 5-tet cube of 0.12 m cells
// (pressure 0 or 300 in turn), both offset by a seeded U[-0.3, 0.3] m in X and Z, so that they land on
// the cap, rim, side and top faces; 5 iterations, `steps` steps of 1/60 s.
inline SceneSpec make_shapes_drop(uint64_t seed = 7, int steps = 150) {
    SceneSpec s;
    Rng rng(seed);
    struct Stand {
        ColliderType type;
        float radius, half_height, top;
    };
    const Stand stands[4] = {{ColliderType::Capsule, 0.4f, 0.5f, 1.8f},
                             {ColliderType::Cylinder, 0.5f, 0.4f, 0.8f},
                             {ColliderType::Cylinder, 0.8f, 0.1f, 0.2f},
                             {ColliderType::Sphere, 0.5f, 0.0f, 1.0f}};
    for (int k = 0; k < 4; ++k) {
        const float x = -4.5f + 3.0f * float(k);
        ColliderSpec c;
        c.type = stands[k].type;
        c.radius = stands[k].radius;
        c.half_extent[1] = stands[k].half_height;
        c.position[0] = x;
        c.position[1] = 0.5f * stands[k].top;
        c.friction = 0.4f;
        c.restitution = 0.1f;
        s.colliders.push_back(c);
        BodySpec cloth;
        cloth.mesh = make_cloth(16, 16, 0.08f, [](uint32_t, uint32_t) { return false; });
        cloth.mesh.attributes = VertexAttributes{1.0e-5f, 1.0e-5f, 1.0e-4f};
        cloth.mesh.bend_type = BendType::Dihedral;
        cloth.position[0] = x + float(rng.uniform() * 0.6 - 0.3);
        cloth.position[1] = stands[k].top + 0.6f;
        cloth.position[2] = float(rng.uniform() * 0.6 - 0.3);
        s.bodies.push_back(cloth);
        BodySpec cube;
        cube.mesh = make_tet_cube(4, 0.12f, 0.0f, 1.0e-6f);
        cube.creation.pressure = (k & 1) ? 300.0f : 0.0f;
        cube.position[0] = x + float(rng.uniform() * 0.6 - 0.3);
        cube.position[1] = stands[k].top + 1.6f;
        cube.position[2] = float(rng.uniform() * 0.6 - 0.3);
        s.bodies.push_back(cube);
    }
    ColliderSpec floor;
    floor.type = ColliderType::Box;
    floor.half_extent[0] = 10.0f;
    floor.half_extent[1] = 1.0f;
    floor.half_extent[2] = 10.0f;
    floor.position[1] = -1.0f;
    s.colliders.push_back(floor);
    s.num_steps = steps;
    return s;
}

// Two-way coupling: three 20 x 20 cloths (0.06 m spacing, 40 g per vertex, dihedral bends) over a static
// floor (top at y = 0). Trampolines A and B have every border vertex pinned at y = 1: a dynamic sphere
// (radius 0.15, 2 kg) falls onto A from 0.5 m above, a dynamic box (half extent 0.12, 2 kg, turned 0.5 rad
// about a tilted axis and spinning) onto B. Cloth C is free and falls onto a static box turned 0.4 rad about Z.
// The rigid bodies move under Jolt's own solver in the reference run; the soft bodies see them through
// each step's colliding shapes. hulls: a fourth cloth falls onto a static irregular convex hull (24
// points on a jittered ellipsoid), and a small dynamic hull drops onto it. `steps` steps of 1/60 s.
// sensors: adds a static box sensor under the first trampoline (it sags into it) and a kinematic sphere
// sensor rising through the second cloth.
inline SceneSpec make_coupling(int steps = 90, bool hulls = false, bool sensors = false) {
    SceneSpec s;
    const float xs[3] = {-1.6f, 0.0f, 1.6f};
    for (int k = 0; k < 3; ++k) {
        BodySpec b;
        const uint32_t n = 20;
        if (k < 2)
            b.mesh = make_cloth(n, n, 0.06f, [n](uint32_t x, uint32_t z) { return x == 0 || z == 0 || x == n - 1 || z == n - 1; });
        else
            b.mesh = make_cloth(n, n, 0.06f, [](uint32_t, uint32_t) { return false; });
        for (float &w : b.mesh.inv_mass)
            if (w > 0.0f) w = 25.0f;  // 40 g per vertex
        b.mesh.attributes = VertexAttributes{1.0e-6f, 1.0e-6f, 1.0e-4f};
        b.mesh.bend_type = BendType::Dihedral;
        b.creation.friction = 0.5f;
        b.position[0] = xs[k];
        b.position[1] = k < 2 ? 1.0f : 1.4f;
        s.bodies.push_back(b);
    }
    RigidSpec floor;
    floor.type = ColliderType::Box;
    floor.motion = 0;
    floor.half_extent[0] = 5.0f;
    floor.half_extent[1] = 0.5f;
    floor.half_extent[2] = 5.0f;
    floor.position[1] = -0.5f;
    s.rigid.push_back(floor);
    RigidSpec ball;
    ball.type = ColliderType::Sphere;
    ball.radius = 0.15f;
    ball.mass = 2.0f;
    ball.friction = 0.4f;
    ball.restitution = 0.2f;
    ball.position[0] = xs[0];
    ball.position[1] = 1.5f;
    s.rigid.push_back(ball);
    RigidSpec box;
    box.type = ColliderType::Box;
    box.half_extent[0] = box.half_extent[1] = box.half_extent[2] = 0.12f;
    box.mass = 2.0f;
    box.friction = 0.6f;
    box.position[0] = xs[1] + 0.05f;
    box.position[1] = 1.5f;
    box.position[2] = -0.04f;
    // 0.5 rad about the unit axis (0.36, 0.48, 0.8)
    const float sh = std::sin(0.25f), ch = std::cos(0.25f);
    box.rotation[0] = 0.36f * sh;
    box.rotation[1] = 0.48f * sh;
    box.rotation[2] = 0.8f * sh;
    box.rotation[3] = ch;
    box.angular_velocity[1] = 2.0f;
    s.rigid.push_back(box);
    RigidSpec ramp;
    ramp.type = ColliderType::Box;
    ramp.motion = 0;
    ramp.half_extent[0] = 0.5f;
    ramp.half_extent[1] = 0.1f;
    ramp.half_extent[2] = 0.5f;
    ramp.position[0] = xs[2];
    ramp.position[1] = 0.5f;
    ramp.rotation[2] = std::sin(0.2f);
    ramp.rotation[3] = std::cos(0.2f);
    ramp.friction = 0.3f;
    s.rigid.push_back(ramp);
    if (hulls) {
        // a fourth cloth (free) falls onto a static irregular convex hull, and a dynamic one drops on top
        BodySpec b;
        const uint32_t n = 20;
        b.mesh = make_cloth(n, n, 0.06f, [](uint32_t, uint32_t) { return false; });
        for (float &w : b.mesh.inv_mass) w = 25.0f;
        b.mesh.attributes = VertexAttributes{1.0e-6f, 1.0e-6f, 1.0e-4f};
        b.mesh.bend_type = BendType::Dihedral;
        b.creation.friction = 0.5f;
        b.position[0] = 3.2f;
        b.position[1] = 1.3f;
        s.bodies.push_back(b);
        Rng rng(11);
        for (int k = 0; k < 2; ++k) {
            RigidSpec h;
            h.type = ColliderType::Hull;
            h.motion = k == 0 ? 0 : 2;
            h.mass = 1.5f;
            h.friction = 0.5f;
            const float scale = k == 0 ? 0.45f : 0.18f;
            for (int i = 0; i < 24; ++i) {  // points on an ellipsoid, jittered
                const double u = rng.uniform() * 2.0 - 1.0, a = rng.uniform() * 6.283185307179586;
                const double r = std::sqrt(1.0 - u * u);
                h.hull_points.push_back({float(scale * 1.3 * r * std::cos(a)), float(scale * 0.8 * u), float(scale * r * std::sin(a))});
            }
            h.position[0] = 3.2f + (k == 0 ? 0.0f : 0.07f);
            h.position[1] = k == 0 ? 0.36f : 2.0f;
            h.position[2] = k == 0 ? 0.0f : -0.05f;
            if (k == 1) {
                h.rotation[0] = std::sin(0.3f);
                h.rotation[3] = std::cos(0.3f);
            }
            s.rigid.push_back(h);
        }
    }
    if (sensors) {
        RigidSpec zone;
        zone.type = ColliderType::Box;
        zone.motion = 0;
        zone.sensor = true;
        zone.half_extent[0] = zone.half_extent[2] = 0.25f;
        zone.half_extent[1] = 0.2f;
        zone.position[0] = xs[0];
        zone.position[1] = 0.75f;
        s.rigid.push_back(zone);
        RigidSpec probe;
        probe.type = ColliderType::Sphere;
        probe.motion = 1;
        probe.sensor = true;
        probe.radius = 0.25f;
        probe.position[0] = xs[1] + 0.1f;
        probe.position[1] = 0.2f;
        probe.velocity[1] = 0.6f;
        s.rigid.push_back(probe);
    }
    s.num_steps = steps;
    return s;
}

}  // namespace scene
}  // namespace jsb
