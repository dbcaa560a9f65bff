// CPU oracle for the soft-body solver step. TEST INFRASTRUCTURE ONLY.
//
// This is a plain restatement of Jolt Physics' soft-body update, written to be checked against the
// reference (oracle/_ref) and then used as the checker of the CUDA path. Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load it. The product library
// (libjsb) never links or calls it.
//
// Threads are used the way the reference's job system uses them, without changing a single operation:
// a world of at least as many bodies as threads steps whole bodies concurrently (bodies do not interact
// within a step); otherwise each body's parallel update groups (vertex-disjoint) run concurrently and
// its non-parallel group runs after them, as ParallelApplyConstraints does
// (SoftBodyMotionProperties.cpp:1057-1115), and the per-vertex passes are split into vertex ranges.
//
// Every arithmetic step follows the reference's operation order so that the float instantiation is
// bit-identical to the reference built with JPH_CROSS_PLATFORM_DETERMINISTIC (-ffp-contract=off):
//   Vec3 dot  = (x*x' + y*y') + (z*z' + 0)          Jolt/Math/Vec3.inl:896-934 (ReduceSum, deterministic)
//   Vec3 cross = separately rounded products         Jolt/Math/Vec3.inl:855-895
//   unary minus = 0 - x                              Jolt/Math/Vec3.inl:669-700
//   Sign(x) = x < 0 ? -1 : 1                         Jolt/Math/Math.h:116-119
//   ACosApproximate                                  Jolt/Math/Trigonometry.h:48-65
// The double instantiation evaluates the same sequence in FP64 ("FP64 re-evaluation").
//
// Step structure (Jolt/Physics/SoftBody/SoftBodyMotionProperties.cpp):
//   InitializeUpdateContext            :937-960
//   DetermineCollidingShapes (broad)   :120-255  (static Box/Sphere colliders, world AABB overlap)
//   DetermineCollisionPlanes           :257-265 + BoxShape.cpp:234-283 + SphereShape.cpp:279-300
//   per iteration: ApplyPressure :291-323, IntegratePositions :325-365,
//                  ProcessGroup for each parallel group, then the non-parallel group :1030-1115
//                  (volume :458-507, dihedral bend :367-456, edge :573-601, LRA :679-698),
//                  ApplyCollisionConstraintsAndUpdateVelocities :700-825 (static-body branch)
//   UpdateSoftBodyState                :827-921
//   body position += delta             Jolt/Physics/PhysicsSystem.cpp:2864
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared oracle/jsb_oracle.cpp -o oracle/liboracle.so

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <limits>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace oracle {

// Persistent workers: run(count, fn) calls fn(i) for every i < count on the workers and the caller,
// and returns when all calls have finished.
class Pool {
public:
    explicit Pool(int threads) {
        for (int t = 1; t < threads; ++t) workers_.emplace_back([this] { loop(); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &w : workers_) w.join();
    }
    int size() const { return int(workers_.size()) + 1; }
    void run(size_t count, const std::function<void(size_t)> &fn) {
        if (workers_.empty() || count < 2) {
            for (size_t i = 0; i < count; ++i) fn(i);
            return;
        }
        {
            std::lock_guard<std::mutex> l(m_);
            fn_ = &fn;
            count_ = count;
            next_.store(0);
            pending_ = int(workers_.size());
            ++generation_;
        }
        cv_.notify_all();
        drain();
        std::unique_lock<std::mutex> l(m_);
        done_cv_.wait(l, [this] { return pending_ == 0; });
        fn_ = nullptr;
    }

private:
    void drain() {
        for (size_t i = next_.fetch_add(1); i < count_; i = next_.fetch_add(1)) (*fn_)(i);
    }
    void loop() {
        size_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return stop_ || generation_ != seen; });
                if (stop_) return;
                seen = generation_;
            }
            drain();
            {
                std::lock_guard<std::mutex> l(m_);
                --pending_;
            }
            done_cv_.notify_one();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(size_t)> *fn_ = nullptr;
    size_t count_ = 0;
    std::atomic<size_t> next_{0};
    size_t generation_ = 0;
    int pending_ = 0;
    bool stop_ = false;
};

template <class R>
struct V3 {
    R x, y, z;
};
template <class R>
inline V3<R> add(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R>
inline V3<R> sub(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R>
inline V3<R> mul(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R>
inline V3<R> mul(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R>
inline V3<R> divs(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R>
inline V3<R> neg(V3<R> a) { return {R(0) - a.x, R(0) - a.y, R(0) - a.z}; }
template <class R>
inline R dot(V3<R> a, V3<R> b) {
    R px = a.x * b.x, py = a.y * b.y, pz = a.z * b.z;
    return (px + py) + (pz + R(0));
}
template <class R>
inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R>
inline R len_sq(V3<R> a) { return dot(a, a); }
template <class R>
inline R len(V3<R> a) { return std::sqrt(len_sq(a)); }
template <class R>
inline R sgn(R v) { return v < R(0) ? R(-1) : R(1); }
template <class R>
inline V3<R> vmin(V3<R> a, V3<R> b) { return {a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z}; }
template <class R>
inline V3<R> vmax(V3<R> a, V3<R> b) { return {a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z}; }
template <class R>
inline R comp(V3<R> a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
template <class R>
inline R acos_approx(R x) {  // Jolt/Math/Trigonometry.h:48-65
    const R pi = R(3.14159265358979323846f);
    R ax = std::abs(x);
    if (ax > R(1)) ax = R(1);
    R val = std::sqrt(R(1) - ax) * (pi / R(2) - R(0.175394f) * ax);
    return x < R(0) ? pi - val : val;
}

// --------------------------------------------------------------------------------------------
// Settings blob (SoftBodySharedSettings::SaveBinaryState, SoftBodySharedSettings.cpp:1203-1236)
// --------------------------------------------------------------------------------------------
struct Edge { uint32_t v[2]; float rest, compliance; };
struct Bend { uint32_t v[4]; float compliance, initial_angle; };
struct Volume { uint32_t v[4]; float six_rest_volume, compliance; };
struct LRA { uint32_t v[2]; float max_distance; };
struct Face { uint32_t v[3]; uint32_t material; };
struct Group { uint32_t edge, lra, rod_ss, rod_bt, bend, volume, skinned; };
struct SVertex { float pos[3], vel[3], inv_mass; };
struct Skinned {  // SoftBodySharedSettings::Skinned
    uint32_t vertex;
    struct { uint32_t inv_bind; float weight; } w[4];
    float max_distance, backstop_distance, backstop_radius;
    uint32_t normal_info;  // start in skinned_normals (low 24 bits), face count (high 8 bits)
};
struct InvBind { uint32_t joint; float m[16]; };  // SoftBodySharedSettings::InvBind, Mat44 columns

struct Settings {
    std::vector<SVertex> vertices;
    std::vector<Face> faces;
    std::vector<Edge> edges;
    std::vector<Bend> bends;
    std::vector<Volume> volumes;
    std::vector<LRA> lras;
    std::vector<Group> groups;
    std::vector<Skinned> skinned;
    std::vector<uint32_t> skinned_normals;
    std::vector<InvBind> inv_binds;
    uint32_t n_skinned = 0, n_rod_ss = 0, n_rod_bt = 0;
};

class Reader {
public:
    Reader(const uint8_t *p, size_t n) : p_(p), n_(n) {}
    bool read(void *dst, size_t bytes) {
        if (off_ + bytes > n_) return false;
        memcpy(dst, p_ + off_, bytes);
        off_ += bytes;
        return true;
    }
    bool skip(size_t bytes) {
        if (off_ + bytes > n_) return false;
        off_ += bytes;
        return true;
    }
    template <class T>
    bool array(std::vector<T> &out, size_t elem_bytes) {
        uint32_t count;
        if (!read(&count, 4)) return false;
        if (uint64_t(count) * elem_bytes > n_ - off_) return false;
        out.resize(count);
        for (uint32_t i = 0; i < count; ++i)
            if (!read(&out[i], elem_bytes)) return false;
        return true;
    }
    bool skip_array(size_t elem_bytes, uint32_t *count_out) {
        uint32_t count;
        if (!read(&count, 4)) return false;
        if (count_out) *count_out = count;
        return skip(uint64_t(count) * elem_bytes);
    }
    size_t offset() const { return off_; }

private:
    const uint8_t *p_;
    size_t n_, off_ = 0;
};

inline bool parse_settings(const uint8_t *blob, size_t len, Settings &s, std::string &err) {
    Reader r(blob, len);
    bool ok = r.array(s.vertices, 28) && r.array(s.faces, 16) && r.array(s.edges, 16) && r.array(s.bends, 24) &&
              r.array(s.volumes, 24) && r.array(s.skinned, 52) && r.array(s.skinned_normals, 4) && r.array(s.lras, 12) &&
              r.array(s.groups, 28) && r.skip_array(36, &s.n_rod_ss) && r.skip_array(28, &s.n_rod_bt) && r.array(s.inv_binds, 68);
    s.n_skinned = uint32_t(s.skinned.size());
    if (!ok) {
        err = "truncated settings blob";
        return false;
    }
    if (r.offset() != len) {
        err = "trailing bytes in settings blob";
        return false;
    }
    return true;
}

// --------------------------------------------------------------------------------------------
// World
// --------------------------------------------------------------------------------------------
struct Collider {
    int type;  // 0 box, 1 sphere
    float pos[3];
    float half[3];
    float radius;
    float friction, restitution;
};

// A colliding shape determined on the host for one body and step (the layout of jsb_colliding_shape):
// the fields of SoftBodyMotionProperties::CollidingShape and its LeafShape the step reads.
struct TableShapeIn {  // 176 bytes
    int32_t type, motion;  // motion: EMotionType (2 = dynamic)
    float xf[12];          // leaf transform: rotation columns 0-2, translation
    float half_extent[3], radius, friction, restitution;
    float inv_mass_scale, inv_mass;
    float inv_inertia[12];  // columns 0-3
    float com[3], lin[3], ang[3];
    uint32_t hull;  // type 4: index of a hull added with oracle_add_hull
};

// A convex hull as ConvexHullShape holds it: points relative to its centre of mass, one plane per face
// (normal, constant), each face's vertex indices.
struct HullData {
    std::vector<float> points;  // 3 per point
    std::vector<float> planes;  // 4 per face
    std::vector<std::vector<uint32_t>> faces;
};

struct Creation {
    uint32_t num_iterations;
    float linear_damping, max_linear_velocity, restitution, friction, pressure, gravity_factor, vertex_radius;
    uint32_t update_position;
    uint32_t allow_sleeping;
};

template <class R>
struct Vertex {
    V3<R> prev, pos, vel;
    R inv_mass;
    V3<R> plane_n;
    R plane_c;
    int shape_idx;
    bool contact;
    R largest_pen;
};

template <class R>
struct Body {
    std::shared_ptr<Settings> settings;
    Creation cs;
    std::vector<Vertex<R>> v;
    V3<R> position;  // body (center of mass) position in world space
    V3<R> bmin, bmax, pmin, pmax;  // local bounds and predicted bounds
    V3<R> force;
    V3<R> lin_vel, ang_vel;
    std::vector<R> edge_c, vol_c;  // per-constraint compliance (the settings' values unless overridden)
    R sleep_timer = R(0);  // MotionProperties::mSleepTestTimer
    bool active = true;    // in the active set (asleep bodies are not stepped)
    // Collision decisions of every step (frozen-decision runs, see World::freeze_mode)
    struct Decisions {
        std::vector<int> shape_collider;  // colliding shapes: collider index, friction, restitution
        std::vector<R> shape_friction, shape_restitution;
        std::vector<int> vertex_shape;  // per vertex: shape index, plane normal and constant (world space:
        std::vector<V3<R>> vertex_n;    // the body position moves with the recentring, the colliders do not)
        std::vector<R> vertex_c;
        std::vector<uint8_t> flags;   // [substep][vertex] bit 0 contact, 1 friction clamped, 2 restitution
        std::vector<uint8_t> vclamp;  // per vertex: velocity clamped after the step
    };
    std::vector<Decisions> decisions;
    size_t decision_step = 0;
    // host-determined colliding shapes (used instead of the world's colliders when has_table), and
    // after a step each shape's {updated, linear velocity, angular velocity}
    bool has_table = false;
    std::vector<TableShapeIn> table;
    std::vector<std::array<float, 7>> table_out;
    // the last step's SoftBodyManifold (World::record_manifold): per vertex {has contact, local contact
    // point, contact normal, shape index}
    std::vector<std::array<float, 8>> manifold;
    uint32_t sensor_hits = 0;  // bit k: table shape k is a sensor shape a vertex penetrated (last step)
    // SkinState per vertex (sized when the settings have skinned constraints) and the skinning switches
    std::vector<V3<R>> skin_prev, skin_pos, skin_normal;
    bool skin_enabled = true, skin_prev_valid = false;
    R skin_mult = R(1);
    uint32_t cur_iteration = 0;  // of the step being run (ApplySkinConstraints' mNextIteration - 1)
};

template <class R>
struct CollidingShape {
    int collider = -1;  // world collider index (-1: host-determined)
    int type = 0;
    V3<R> t;  // translation relative to the soft body
    V3<R> h;  // half extent (capsule / cylinder: h.y = half height)
    R r = R(0);
    R friction, restitution;
    R isc = R(1);  // mSoftBodyInvMassScale
    bool rotated = false, dynamic = false;
    bool sensor = false;  // a sensor's leaf shape (CollidingSensor): no collision plane, only a contact test
    const HullData *hull = nullptr;  // type 4
    V3<R> c[3], ic[3], it;  // rotation columns; Mat44::InversedRotationTranslation columns and translation
    R inv_mass = R(0);
    V3<R> inertia[4];  // mInvInertia columns 0-3
    V3<R> com, lin, ang;
    bool updated = false;
};

// Mat44 * Vec3 (Mat44.inl:295-302) and Mat44::Multiply3x3 (:384-390) over columns
template <class R>
inline V3<R> mat3(const V3<R> c[3], V3<R> v) {
    return {(c[0].x * v.x + c[1].x * v.y) + c[2].x * v.z, (c[0].y * v.x + c[1].y * v.y) + c[2].y * v.z,
            (c[0].z * v.x + c[1].z * v.y) + c[2].z * v.z};
}
template <class R>
inline V3<R> mat4(const V3<R> c[3], V3<R> t, V3<R> v) {
    V3<R> m = mat3(c, v);
    return {m.x + t.x, m.y + t.y, m.z + t.z};
}

template <class R>
class World {
public:
    const std::vector<HullData> *hulls = nullptr;  // the handle's registered hulls
    bool record_manifold = false;
    V3<R> gravity{R(0), R(-9.81f), R(0)};
    std::vector<Collider> colliders;
    std::vector<Body<R>> bodies;

    int add_body(std::shared_ptr<Settings> s, const float pos[3], const Creation &cs) {
        Body<R> b;
        b.settings = s;
        b.cs = cs;
        b.position = {R(pos[0]), R(pos[1]), R(pos[2])};
        b.force = {R(0), R(0), R(0)};
        b.lin_vel = b.ang_vel = {R(0), R(0), R(0)};
        const R big = R(FLT_MAX);
        b.bmin = {big, big, big};
        b.bmax = {-big, -big, -big};
        b.v.resize(s->vertices.size());
        if (!s->skinned.empty()) {
            const V3<R> z = {R(0), R(0), R(0)};
            b.skin_prev.assign(s->vertices.size(), z);
            b.skin_pos.assign(s->vertices.size(), z);
            b.skin_normal.assign(s->vertices.size(), z);
        }
        for (const Edge &e : s->edges) b.edge_c.push_back(R(e.compliance));
        for (const Volume &vol : s->volumes) b.vol_c.push_back(R(vol.compliance));
        for (size_t i = 0; i < s->vertices.size(); ++i) {  // SoftBodyMotionProperties::Initialize :59-105
            const SVertex &sv = s->vertices[i];
            Vertex<R> &o = b.v[i];
            o.pos = o.prev = {R(sv.pos[0]), R(sv.pos[1]), R(sv.pos[2])};
            o.vel = {R(sv.vel[0]), R(sv.vel[1]), R(sv.vel[2])};
            o.inv_mass = R(sv.inv_mass);
            reset_collision(o);
            b.bmin = vmin(b.bmin, o.pos);
            b.bmax = vmax(b.bmax, o.pos);
        }
        b.pmin = b.bmin;
        b.pmax = b.bmax;
        bodies.push_back(std::move(b));
        return int(bodies.size()) - 1;
    }

    static void reset_collision(Vertex<R> &o) {
        o.largest_pen = R(-FLT_MAX);
        o.shape_idx = -1;
        o.contact = false;
    }

    int threads = 1;
    R time_before_sleep = R(0.5f), sleep_velocity_threshold = R(0.03f);  // PhysicsSettings.h:95,102
    // Frozen-decision runs (TEST INFRASTRUCTURE for finite differences of what the adjoint differentiates):
    // 1 = record every collision decision of every step (colliding shapes, each vertex's plane and shape,
    // per substep contact, friction clamp and restitution, the velocity clamp); 2 = replay them instead
    // of deciding again, with the planes as constants, so that a perturbed run follows the base run's
    // collision active set. 0 = the reference's arithmetic.
    int freeze_mode = 0;
    std::unique_ptr<Pool> pool;
    Pool *inner = nullptr;  // set while one body is stepped with its groups spread over the pool

    // Bodies are independent within a step: with at least as many bodies as threads they are stepped
    // concurrently, one body per task; otherwise one after another, each spreading its parallel update
    // groups and per-vertex passes over the threads. Each body's arithmetic is unchanged either way.
    void step(R dt, int collision_steps) {
        R step_dt = dt / R(collision_steps);
        if (threads > 1 && (!pool || pool->size() != threads)) pool.reset(new Pool(threads));
        for (int c = 0; c < collision_steps; ++c) {
            if (threads <= 1) {
                for (auto &b : bodies) step_body(b, step_dt);
            } else if (bodies.size() >= size_t(threads)) {
                pool->run(bodies.size(), [&](size_t i) { step_body(bodies[i], step_dt); });
            } else {
                inner = pool.get();
                for (auto &b : bodies) step_body(b, step_dt);
                inner = nullptr;
            }
        }
    }

    // fn(first, last) over vertex ranges of a body (on the pool when one body is spread over it)
    template <class F>
    void for_vertex_ranges(size_t n, F &&fn) {
        const size_t chunk = 4096;
        if (!inner || n <= chunk) {
            fn(size_t(0), n);
            return;
        }
        inner->run((n + chunk - 1) / chunk, [&](size_t k) { fn(k * chunk, std::min(n, (k + 1) * chunk)); });
    }

    void step_body(Body<R> &b, R dt) {
        if (!b.active) return;  // asleep: PhysicsSystem steps only active soft bodies (PhysicsSystem.cpp:2711-2716)
        const Settings &s = *b.settings;
        // InitializeUpdateContext (:937-960), identity body rotation
        V3<R> g = mul(R(b.cs.gravity_factor), gravity);
        const uint32_t n_it = b.cs.num_iterations;
        R dt_sub = dt / R(float(n_it));
        R disp_scale = R(0.5f) * R(float(n_it));
        disp_scale = disp_scale * R(float(n_it + 1));
        disp_scale = disp_scale * (dt_sub * dt_sub);
        V3<R> disp_g = mul(disp_scale, g);

        // DetermineCollidingShapes (:120-255)
        std::vector<CollidingShape<R>> shapes;
        typename Body<R>::Decisions *dec = nullptr;
        if (freeze_mode == 1) {
            b.decisions.emplace_back();
            dec = &b.decisions.back();
        } else if (freeze_mode == 2) {
            dec = &b.decisions[b.decision_step++];
            for (size_t k = 0; k < dec->shape_collider.size(); ++k) {
                CollidingShape<R> cs;
                cs.collider = dec->shape_collider[k];
                const Collider &c = colliders[size_t(cs.collider)];
                set_shape_geometry(cs, c);
                cs.t = sub(V3<R>{R(c.pos[0]), R(c.pos[1]), R(c.pos[2])}, b.position);
                cs.friction = dec->shape_friction[k];
                cs.restitution = dec->shape_restitution[k];
                shapes.push_back(cs);
            }
        }
        if (b.has_table) {
            shapes_from_table(b, shapes);
        } else if (freeze_mode != 2) {
            V3<R> lmin = vmin(b.bmin, b.pmin), lmax = vmax(b.bmax, b.pmax);
            V3<R> r3 = {R(b.cs.vertex_radius), R(b.cs.vertex_radius), R(b.cs.vertex_radius)};
            lmin = sub(lmin, r3);
            lmax = add(lmax, r3);
            V3<R> wmin = add(b.position, lmin), wmax = add(b.position, lmax);
            for (size_t ci = 0; ci < colliders.size(); ++ci) {
                const Collider &c = colliders[ci];
                V3<R> cp = {R(c.pos[0]), R(c.pos[1]), R(c.pos[2])};
                // world bounds of the shape (Shape::GetWorldSpaceBounds; CapsuleShape.cpp:266-276)
                V3<R> cmin, cmax;
                if (c.type == 2) {
                    V3<R> rr = {R(c.radius), R(c.radius), R(c.radius)};
                    cmin = sub(V3<R>{cp.x, cp.y - R(c.half[1]), cp.z}, rr);
                    cmax = add(V3<R>{cp.x, cp.y + R(c.half[1]), cp.z}, rr);
                } else {
                    V3<R> ext = c.type == 0   ? V3<R>{R(c.half[0]), R(c.half[1]), R(c.half[2])}
                                : c.type == 1 ? V3<R>{R(c.radius), R(c.radius), R(c.radius)}
                                              : V3<R>{R(c.radius), R(c.half[1]), R(c.radius)};
                    cmin = add(cp, neg(ext));
                    cmax = add(cp, ext);
                }
                bool overlap = !(wmin.x > cmax.x || wmin.y > cmax.y || wmin.z > cmax.z || wmax.x < cmin.x || wmax.y < cmin.y ||
                                 wmax.z < cmin.z);
                if (!overlap) continue;
                CollidingShape<R> cs;
                cs.collider = int(ci);
                set_shape_geometry(cs, c);
                cs.t = sub(cp, b.position);
                cs.friction = std::sqrt(R(b.cs.friction) * R(c.friction));
                cs.restitution = R(b.cs.restitution) > R(c.restitution) ? R(b.cs.restitution) : R(c.restitution);
                shapes.push_back(cs);
                if (dec) {
                    dec->shape_collider.push_back(cs.collider);
                    dec->shape_friction.push_back(cs.friction);
                    dec->shape_restitution.push_back(cs.restitution);
                }
            }
        }

        // DetermineSensorCollisions (:267-289): one penetration shared by all vertices of a sensor shape,
        // a contact when the largest is positive
        b.sensor_hits = 0;
        for (size_t si = 0; si < shapes.size(); ++si) {
            const CollidingShape<R> &cs = shapes[si];
            if (!cs.sensor) continue;
            for (const auto &v : b.v) {
                if (!(v.inv_mass > R(0))) continue;
                Vertex<R> t = v;
                t.largest_pen = R(-FLT_MAX);
                collide_one(t, cs, int(si));
                if (t.largest_pen > R(0)) {
                    b.sensor_hits |= 1u << si;
                    break;
                }
            }
        }

        // DetermineCollisionPlanes (:257-265)
        for (size_t si = 0; si < shapes.size() && freeze_mode != 2; ++si) {
            const CollidingShape<R> &cs = shapes[si];
            if (cs.sensor) continue;
            for (auto &v : b.v) {
                if (!(v.inv_mass > R(0))) continue;
                if (cs.type == 4)
                    collide_hull(v, cs, int(si));
                else if (cs.type == 0)
                    collide_box(v, cs, int(si));
                else if (cs.type == 1)
                    collide_sphere(v, cs, int(si));
                else if (cs.type == 2)
                    collide_capsule(v, cs, int(si));
                else
                    collide_cylinder(v, cs, int(si));
            }
        }

        if (freeze_mode == 2) {
            for (size_t i = 0; i < b.v.size(); ++i) {
                b.v[i].shape_idx = dec->vertex_shape[i];
                b.v[i].plane_n = dec->vertex_n[i];
                b.v[i].plane_c = dec->vertex_c[i] + dot(dec->vertex_n[i], b.position);
            }
        } else if (dec) {
            for (const Vertex<R> &v : b.v) {
                dec->vertex_shape.push_back(v.shape_idx);
                dec->vertex_n.push_back(v.plane_n);
                dec->vertex_c.push_back(v.plane_c - dot(v.plane_n, b.position));
            }
            dec->flags.assign(size_t(n_it) * b.v.size(), 0);
            dec->vclamp.assign(b.v.size(), 0);
        }
        for (uint32_t it = 0; it < n_it; ++it) {
            b.cur_iteration = it;
            apply_pressure(b, dt_sub);
            integrate(b, g, dt_sub);
            const size_t ng = s.groups.size();
            if (inner && ng > 2) {
                // the parallel groups touch disjoint vertices; the last (non-parallel) group follows them
                inner->run(ng - 1, [&](size_t gi) { process_group(b, gi, dt_sub); });
                process_group(b, ng - 1, dt_sub);
            } else {
                for (size_t gi = 0; gi < ng; ++gi) process_group(b, gi, dt_sub);
            }
            collide_and_update_velocities(b, shapes, g, dt_sub, dec ? dec->flags.data() + size_t(it) * b.v.size() : nullptr);
        }
        update_state(b, dt, disp_g, dec);
        if (b.has_table) {
            b.table_out.assign(shapes.size(), {});
            for (size_t k = 0; k < shapes.size(); ++k)
                b.table_out[k] = {shapes[k].updated ? 1.0f : 0.0f, float(shapes[k].lin.x), float(shapes[k].lin.y), float(shapes[k].lin.z),
                                  float(shapes[k].ang.x), float(shapes[k].ang.y), float(shapes[k].ang.z)};
        }
    }

    static void set_shape_geometry(CollidingShape<R> &cs, const Collider &c) {
        cs.type = c.type;
        cs.h = {R(c.half[0]), R(c.half[1]), R(c.half[2])};
        cs.r = R(c.radius);
    }

    // Host-determined shapes (oracle_set_colliding_shapes), with the inverse transform as
    // Mat44::InversedRotationTranslation computes it: transposed rotation, 0 - (R^T t).
    void shapes_from_table(const Body<R> &b, std::vector<CollidingShape<R>> &shapes) const {
        for (const TableShapeIn &e : b.table) {
            CollidingShape<R> cs;
            cs.type = e.type;
            if (e.type == 4) cs.hull = &(*hulls)[e.hull];
            cs.rotated = true;
            cs.dynamic = e.motion == 2;
            cs.sensor = e.motion == 3;
            for (int k = 0; k < 3; ++k) cs.c[k] = {R(e.xf[3 * k]), R(e.xf[3 * k + 1]), R(e.xf[3 * k + 2])};
            for (int k = 0; k < 3; ++k) cs.ic[k] = {comp(cs.c[0], k), comp(cs.c[1], k), comp(cs.c[2], k)};
            cs.t = {R(e.xf[9]), R(e.xf[10]), R(e.xf[11])};
            cs.it = neg(mat3(cs.ic, cs.t));
            cs.h = {R(e.half_extent[0]), R(e.half_extent[1]), R(e.half_extent[2])};
            cs.r = R(e.radius);
            cs.friction = R(e.friction);
            cs.restitution = R(e.restitution);
            cs.isc = R(e.inv_mass_scale);
            cs.inv_mass = R(e.inv_mass);
            for (int k = 0; k < 4; ++k) cs.inertia[k] = {R(e.inv_inertia[3 * k]), R(e.inv_inertia[3 * k + 1]), R(e.inv_inertia[3 * k + 2])};
            cs.com = {R(e.com[0]), R(e.com[1]), R(e.com[2])};
            cs.lin = {R(e.lin[0]), R(e.lin[1]), R(e.lin[2])};
            cs.ang = {R(e.ang[0]), R(e.ang[1]), R(e.ang[2])};
            shapes.push_back(cs);
        }
    }

    static void collide_one(Vertex<R> &v, const CollidingShape<R> &cs, int idx) {
        if (cs.type == 4)
            collide_hull(v, cs, idx);
        else if (cs.type == 0)
            collide_box(v, cs, idx);
        else if (cs.type == 1)
            collide_sphere(v, cs, idx);
        else if (cs.type == 2)
            collide_capsule(v, cs, idx);
        else
            collide_cylinder(v, cs, idx);
    }

    // The shape's CollideSoftBodyVertices maps the vertex with its InversedRotationTranslation ...
    static V3<R> local_of(const CollidingShape<R> &cs, V3<R> p) { return cs.rotated ? mat4(cs.ic, cs.it, p) : add(p, neg(cs.t)); }
    // ... and stores Plane::sFromPointAndNormal(point, normal).GetTransformed(transform) (Plane.h:42-46)
    static void set_plane(Vertex<R> &v, const CollidingShape<R> &cs, V3<R> normal, V3<R> point, int idx) {
        if (!cs.rotated) {
            set_plane_transformed(v, normal, point, cs.t, idx);
            return;
        }
        R c = -dot(normal, point);
        V3<R> n2 = mat3(cs.c, normal);
        v.plane_n = n2;
        v.plane_c = c - dot(cs.t, n2);
        v.shape_idx = idx;
    }

    static void collide_box(Vertex<R> &v, const CollidingShape<R> &cs, int idx) {  // BoxShape.cpp:234-283
        V3<R> local = local_of(cs, v.pos);
        V3<R> h = cs.h;
        V3<R> nh = neg(h);
        V3<R> clamped = vmax(vmin(local, h), nh);
        if (clamped.x == local.x && clamped.y == local.y && clamped.z == local.z) {
            V3<R> al = {std::abs(local.x), std::abs(local.y), std::abs(local.z)};
            V3<R> delta = sub(h, al);
            int index = delta.x < delta.y ? (delta.z < delta.x ? 2 : 0) : (delta.z < delta.y ? 2 : 1);
            R pen = comp(delta, index);
            if (v.largest_pen >= pen) return;
            v.largest_pen = pen;
            V3<R> sign = {std::signbit(local.x) ? R(-1) : R(1), std::signbit(local.y) ? R(-1) : R(1), std::signbit(local.z) ? R(-1) : R(1)};
            V3<R> axis = {index == 0 ? R(1) : R(0), index == 1 ? R(1) : R(0), index == 2 ? R(1) : R(0)};
            V3<R> normal = {sign.x * axis.x, sign.y * axis.y, sign.z * axis.z};
            V3<R> point = {normal.x * h.x, normal.y * h.y, normal.z * h.z};
            set_plane(v, cs, normal, point, idx);
        } else {
            V3<R> normal = sub(local, clamped);
            R nl = len(normal);
            R pen = -nl;
            if (v.largest_pen >= pen) return;
            v.largest_pen = pen;
            normal = divs(normal, nl);
            set_plane(v, cs, normal, clamped, idx);
        }
    }

    // Plane::sFromPointAndNormal(point, normal).GetTransformed(translation t, identity rotation)
    static void set_plane_transformed(Vertex<R> &v, V3<R> normal, V3<R> point, V3<R> t, int idx) {
        R c = -dot(normal, point);
        // Multiply3x3 with identity columns: ((c0*x + c1*y) + c2*z)
        V3<R> n2;
        n2.x = (R(1) * normal.x + R(0) * normal.y) + R(0) * normal.z;
        n2.y = (R(0) * normal.x + R(1) * normal.y) + R(0) * normal.z;
        n2.z = (R(0) * normal.x + R(0) * normal.y) + R(1) * normal.z;
        v.plane_n = n2;
        v.plane_c = c - dot(t, n2);
        v.shape_idx = idx;
    }

    static void collide_sphere(Vertex<R> &v, const CollidingShape<R> &cs, int idx) {  // SphereShape.cpp:279-300
        V3<R> center = cs.t;
        R radius = cs.r;
        V3<R> delta = sub(v.pos, center);
        R distance = len(delta);
        R pen = radius - distance;
        if (v.largest_pen >= pen) return;
        v.largest_pen = pen;
        V3<R> normal = distance > R(0) ? divs(delta, distance) : V3<R>{R(0), R(1), R(0)};
        V3<R> point = add(center, mul(radius, normal));
        v.plane_n = normal;
        v.plane_c = -dot(normal, point);
        v.shape_idx = idx;
    }

    // CapsuleShape.cpp:324-374: along Y, half[1] = half height of the cylinder part
    static void collide_capsule(Vertex<R> &v, const CollidingShape<R> &cs, int idx) {
        const V3<R> local = local_of(cs, v.pos);
        const R hh = cs.h.y, r = cs.r;
        if (std::abs(local.y) <= hh) {
            V3<R> normal = {local.x, R(0), local.z};
            const R nl = len(normal);
            const R pen = r - nl;
            if (v.largest_pen >= pen) return;
            v.largest_pen = pen;
            normal = nl > R(0) ? divs(normal, nl) : V3<R>{R(1), R(0), R(0)};
            set_plane(v, cs, normal, mul(r, normal), idx);
        } else {
            const V3<R> center = {R(0), (local.y < R(0) ? R(-1) : R(1)) * hh, R(0)};
            const V3<R> delta = sub(local, center);
            const R distance = len(delta);
            const R pen = r - distance;
            if (v.largest_pen >= pen) return;
            v.largest_pen = pen;
            const V3<R> normal = divs(delta, distance);
            set_plane(v, cs, normal, add(center, mul(r, normal)), idx);
        }
    }

    // ClosestPoint::GetClosestPointOnLine (Jolt/Geometry/ClosestPoint.h:15-43, 129-150)
    static V3<R> closest_point_on_line(V3<R> a, V3<R> b) {
        const V3<R> ab = sub(b, a);
        const R den = len_sq(ab);
        R u, v;
        const R eps = R(FLT_EPSILON * FLT_EPSILON);
        if (den < eps) {
            const bool a_closer = len_sq(a) < len_sq(b);
            u = a_closer ? R(1) : R(0);
            v = a_closer ? R(0) : R(1);
        } else {
            v = -dot(a, ab) / den;
            u = R(1) - v;
        }
        if (v <= R(0)) return a;
        if (u <= R(0)) return b;
        return add(mul(u, a), mul(v, b));
    }

    // ConvexHullShape.cpp:1060-1163, unscaled
    static void collide_hull(Vertex<R> &v, const CollidingShape<R> &cs, int idx) {
        const HullData &h = *cs.hull;
        const V3<R> local = local_of(cs, v.pos);
        R max_distance = -R(FLT_MAX);
        V3<R> max_n = {R(0), R(0), R(0)};
        size_t max_i = 0;
        const size_t nf = h.planes.size() / 4;
        for (size_t i = 0; i < nf; ++i) {
            const V3<R> n = {R(h.planes[4 * i]), R(h.planes[4 * i + 1]), R(h.planes[4 * i + 2])};
            const R distance = dot(local, n) + R(h.planes[4 * i + 3]);
            if (distance > max_distance) {
                max_distance = distance;
                max_n = n;
                max_i = i;
            }
        }
        V3<R> closest = mul(-max_distance, max_n);
        const bool outside = max_distance > R(0);
        if (outside) {
            R best = R(FLT_MAX);
            const std::vector<uint32_t> &face = h.faces[max_i];
            for (size_t k = 0; k < face.size(); ++k) {
                const uint32_t a = face[k], b = face[k + 1 == face.size() ? 0 : k + 1];
                const V3<R> p1 = {R(h.points[3 * a]), R(h.points[3 * a + 1]), R(h.points[3 * a + 2])};
                const V3<R> p2 = {R(h.points[3 * b]), R(h.points[3 * b + 1]), R(h.points[3 * b + 2])};
                if (dot(cross(sub(p2, p1), max_n), sub(local, p1)) > R(0)) {
                    const V3<R> c = closest_point_on_line(sub(p1, local), sub(p2, local));
                    const R dsq = len_sq(c);
                    if (dsq < best) {
                        best = dsq;
                        closest = c;
                    }
                }
            }
        }
        V3<R> normal = neg(closest);
        const R nl = len(normal);
        R pen = nl;
        if (outside)
            pen = -pen;
        else
            normal = neg(normal);
        if (v.largest_pen >= pen) return;
        v.largest_pen = pen;
        normal = nl > R(1.0e-12f) ? divs(normal, nl) : max_n;
        set_plane(v, cs, normal, add(local, closest), idx);
    }

    // CylinderShape.cpp:317-368: along Y, half[1] = half height
    static void collide_cylinder(Vertex<R> &v, const CollidingShape<R> &cs, int idx) {
        const V3<R> local = local_of(cs, v.pos);
        const R hh = cs.h.y, r = cs.r;
        const V3<R> side = {local.x, R(0), local.z};
        const R side_len = len(side);
        const R side_pen = r - side_len;
        const R top_pen = hh - std::abs(local.y);
        const R sgn = local.y < R(0) ? R(-1) : R(1);
        V3<R> point, normal;
        if (side_pen < R(0) && top_pen < R(0)) {
            point = add(mul(side, r / side_len), V3<R>{R(0), hh * sgn, R(0)});
            const V3<R> d = sub(local, point);
            const R px = d.x * d.x, py = d.y * d.y, pz = d.z * d.z;
            const R lsq = (px + py) + pz;  // Vec3::NormalizedOr (Vec3.inl:978-998)
            const R tiny = R(std::numeric_limits<float>::min());
            normal = lsq <= tiny ? V3<R>{R(0), R(1), R(0)} : divs(d, std::sqrt(lsq));
        } else if (side_pen < top_pen) {
            normal = side_len > R(0) ? divs(side, side_len) : V3<R>{R(1), R(0), R(0)};
            point = mul(r, normal);
        } else {
            normal = {R(0), sgn, R(0)};
            point = mul(hh, normal);
        }
        const R cst = -dot(normal, point);
        const R pen = -(dot(local, normal) + cst);
        if (v.largest_pen >= pen) return;
        v.largest_pen = pen;
        set_plane(v, cs, normal, point, idx);
    }

    void apply_pressure(Body<R> &b, R dt) {  // :291-323
        R pc = R(b.cs.pressure);
        if (!(pc > R(0))) return;
        const Settings &s = *b.settings;
        R six_volume = R(0);
        for (const Face &f : s.faces) {
            V3<R> x1 = b.v[f.v[0]].pos, x2 = b.v[f.v[1]].pos, x3 = b.v[f.v[2]].pos;
            six_volume = six_volume + dot(cross(x1, x2), x3);
        }
        if (!(six_volume > R(0))) return;
        R coefficient = pc * dt / six_volume;
        for (const Face &f : s.faces) {
            V3<R> x1 = b.v[f.v[0]].pos, x2 = b.v[f.v[1]].pos, x3 = b.v[f.v[2]].pos;
            V3<R> impulse = mul(coefficient, cross(sub(x2, x1), sub(x3, x1)));
            for (int k = 0; k < 3; ++k) {
                Vertex<R> &vv = b.v[f.v[k]];
                vv.vel = add(vv.vel, mul(vv.inv_mass, impulse));
            }
        }
    }

    void integrate(Body<R> &b, V3<R> g, R dt) {  // :325-365
        R damp = R(1) - R(b.cs.linear_damping) * dt;
        if (damp < R(0)) damp = R(0);
        V3<R> sub_g = mul(g, dt);
        R nv = R(float(b.v.size() > 0 ? b.v.size() : 1));
        V3<R> sub_imp = divs(mul(b.force, dt), nv);
        for_vertex_ranges(b.v.size(), [&](size_t first, size_t last) {
            for (size_t i = first; i < last; ++i) {
                Vertex<R> &v = b.v[i];
                if (v.inv_mass > R(0)) {
                    v.vel = add(v.vel, add(sub_g, mul(sub_imp, v.inv_mass)));
                    v.vel = mul(v.vel, damp);
                }
                V3<R> p = v.pos;
                v.prev = p;
                v.pos = add(p, mul(v.vel, dt));
            }
        });
    }

    void process_group(Body<R> &b, size_t gi, R dt) {  // :1030-1055
        const Settings &s = *b.settings;
        Group start{0, 0, 0, 0, 0, 0, 0};
        const Group &prev = gi > 0 ? s.groups[gi - 1] : start;
        const Group &cur = s.groups[gi];
        R inv_dt_sq = R(1) / (dt * dt);
        for (uint32_t i = prev.volume; i < cur.volume; ++i) apply_volume(b, s.volumes[i], b.vol_c[i], inv_dt_sq);
        for (uint32_t i = prev.bend; i < cur.bend; ++i) apply_bend(b, s.bends[i], inv_dt_sq);
        for (uint32_t i = prev.skinned; i < cur.skinned; ++i) apply_skin(b, s.skinned[i]);
        for (uint32_t i = prev.edge; i < cur.edge; ++i) apply_edge(b, s.edges[i], b.edge_c[i], inv_dt_sq);
        for (uint32_t i = prev.lra; i < cur.lra; ++i) apply_lra(b, s.lras[i]);
    }

    void apply_skin(Body<R> &b, const Skinned &sk) {  // ApplySkinConstraints :509-571
        if (!b.skin_enabled) return;
        const R factor = b.skin_prev_valid ? R(float(b.cur_iteration + 1)) / R(float(b.cs.num_iterations)) : R(1);
        const R prev_factor = R(1) - factor;
        Vertex<R> &v = b.v[sk.vertex];
        const R max_distance = R(sk.max_distance) * b.skin_mult;
        const V3<R> skin_pos = add(mul(prev_factor, b.skin_prev[sk.vertex]), mul(factor, b.skin_pos[sk.vertex]));
        if (max_distance > R(0)) {
            const R bsd = R(sk.backstop_distance), bsr = R(sk.backstop_radius);
            if (bsd < max_distance) {
                const V3<R> n = b.skin_normal[sk.vertex];
                const V3<R> center = sub(skin_pos, mul(bsd + bsr, n));
                const V3<R> delta = sub(v.pos, center);
                const R dls = len_sq(delta);
                if (dls < bsr * bsr) {
                    const R dl = std::sqrt(dls);
                    v.pos = dl > R(0) ? add(center, mul(bsr / dl, delta)) : add(center, mul(bsr, n));
                }
            }
            if (max_distance < R(FLT_MAX)) {
                const V3<R> delta = sub(v.pos, skin_pos);
                const R dls = len_sq(delta);
                const R mds = max_distance * max_distance;
                if (dls > mds) v.pos = add(skin_pos, mul(std::sqrt(mds / dls), delta));
            }
        } else {
            v.pos = skin_pos;
        }
    }

    // SkinVertices (:1139-1230) with joint matrices (16 floats each, Mat44 columns): Mat44 * Mat44 and
    // Mat44 * Vec3 as ((c0 x + c1 y) + c2 z) + c3 (Mat44.inl:241-302).
    void skin_vertices(Body<R> &b, const float *joints, uint32_t nj, bool hard) {
        const Settings &s = *b.settings;
        std::vector<std::array<R, 16>> mats(s.inv_binds.size());
        for (size_t k = 0; k < mats.size(); ++k) {
            const float *J = joints + 16 * size_t(s.inv_binds[k].joint);
            const float *M = s.inv_binds[k].m;
            for (int i = 0; i < 4; ++i)
                for (int r = 0; r < 4; ++r)
                    mats[k][4 * i + r] = ((R(J[r]) * R(M[4 * i]) + R(J[4 + r]) * R(M[4 * i + 1])) + R(J[8 + r]) * R(M[4 * i + 2])) +
                                         R(J[12 + r]) * R(M[4 * i + 3]);
        }
        (void)nj;
        for (const Skinned &sk : s.skinned) {
            const SVertex &bv = s.vertices[sk.vertex];
            const R bx = R(bv.pos[0]), by = R(bv.pos[1]), bz = R(bv.pos[2]);
            V3<R> pos = {R(0), R(0), R(0)};
            for (const auto &w : sk.w) {
                if (w.weight == 0.0f) break;
                const auto &m = mats[w.inv_bind];
                V3<R> mv;
                mv.x = ((m[0] * bx + m[4] * by) + m[8] * bz) + m[12];
                mv.y = ((m[1] * bx + m[5] * by) + m[9] * bz) + m[13];
                mv.z = ((m[2] * bx + m[6] * by) + m[10] * bz) + m[14];
                pos = add(pos, mul(R(w.weight), mv));
            }
            b.skin_prev[sk.vertex] = b.skin_pos[sk.vertex];
            b.skin_pos[sk.vertex] = pos;
        }
        auto normalized_or_zero = [](V3<R> v) {
            const R l2 = (v.x * v.x + v.y * v.y) + v.z * v.z;
            if (l2 <= R(FLT_MIN)) return V3<R>{R(0), R(0), R(0)};
            const R l = std::sqrt(l2);
            return V3<R>{v.x / l, v.y / l, v.z / l};
        };
        for (const Skinned &sk : s.skinned) {
            V3<R> n = {R(0), R(0), R(0)};
            const uint32_t nf = sk.normal_info >> 24;
            if (nf > 0) {
                for (uint32_t k = 0; k < nf; ++k) {
                    const Face &f = s.faces[s.skinned_normals[(sk.normal_info & 0xffffffu) + k]];
                    const V3<R> v0 = b.skin_pos[f.v[0]], v1 = b.skin_pos[f.v[1]], v2 = b.skin_pos[f.v[2]];
                    n = add(n, normalized_or_zero(cross(sub(v1, v0), sub(v2, v0))));
                }
                n = normalized_or_zero(n);
            }
            b.skin_normal[sk.vertex] = n;
        }
        if (hard) {
            for (const Skinned &sk : s.skinned) {
                b.skin_prev[sk.vertex] = b.skin_pos[sk.vertex];
                b.v[sk.vertex].pos = b.skin_pos[sk.vertex];
                b.v[sk.vertex].vel = {R(0), R(0), R(0)};
            }
        } else if (!b.skin_enabled) {
            for (const Skinned &sk : s.skinned)
                if (sk.max_distance == 0.0f) b.v[sk.vertex].pos = b.skin_pos[sk.vertex];
        }
        b.skin_prev_valid = true;
    }

    void apply_bend(Body<R> &b, const Bend &c, R inv_dt_sq) {  // :367-456
        Vertex<R> &v0 = b.v[c.v[0]], &v1 = b.v[c.v[1]], &v2 = b.v[c.v[2]], &v3 = b.v[c.v[3]];
        V3<R> x0 = v0.pos, x1 = v1.pos, x2 = v2.pos, x3 = v3.pos;
        V3<R> e = sub(x1, x0);
        R e_len = len(e);
        if (e_len < R(1.0e-6f)) return;
        V3<R> x1x2 = sub(x2, x1), x1x3 = sub(x3, x1);
        V3<R> n1 = cross(sub(x2, x0), x1x2);
        V3<R> n2 = cross(x1x3, sub(x3, x0));
        R n1_len_sq = len_sq(n1), n2_len_sq = len_sq(n2);
        R n1n2 = n1_len_sq * n2_len_sq;
        if (n1n2 < R(1.0e-24f)) return;
        R sign = sgn(dot(cross(n2, n1), e));
        R d = dot(n1, n2) / std::sqrt(n1n2);
        const R pi = R(3.14159265358979323846f);
        R cval = sign * acos_approx(d) - R(c.initial_angle);
        if (cval > pi)
            cval -= R(2.0f) * pi;
        else if (cval < -pi)
            cval += R(2.0f) * pi;
        n1 = divs(n1, n1_len_sq);
        n2 = divs(n2, n2_len_sq);
        V3<R> d0c = divs(add(mul(dot(x1x2, e), n1), mul(dot(x1x3, e), n2)), e_len);
        V3<R> d2c = mul(e_len, n1);
        V3<R> d3c = mul(e_len, n2);
        V3<R> d1c = sub(sub(neg(d0c), d2c), d3c);
        R w0 = v0.inv_mass, w1 = v1.inv_mass, w2 = v2.inv_mass, w3 = v3.inv_mass;
        R denom = w0 * len_sq(d0c) + w1 * len_sq(d1c) + w2 * len_sq(d2c) + w3 * len_sq(d3c) + R(c.compliance) * inv_dt_sq;
        if (denom < R(1.0e-12f)) return;
        R ml = cval / denom;
        v0.pos = sub(x0, mul(ml * w0, d0c));
        v1.pos = sub(x1, mul(ml * w1, d1c));
        v2.pos = sub(x2, mul(ml * w2, d2c));
        v3.pos = sub(x3, mul(ml * w3, d3c));
    }

    void apply_volume(Body<R> &b, const Volume &c, R compliance, R inv_dt_sq) {  // :458-507
        Vertex<R> &v1 = b.v[c.v[0]], &v2 = b.v[c.v[1]], &v3 = b.v[c.v[2]], &v4 = b.v[c.v[3]];
        V3<R> x1 = v1.pos, x2 = v2.pos, x3 = v3.pos, x4 = v4.pos;
        V3<R> x1x2 = sub(x2, x1), x1x3 = sub(x3, x1), x1x4 = sub(x4, x1);
        R cval = std::abs(dot(cross(x1x2, x1x3), x1x4)) - R(c.six_rest_volume);
        V3<R> d1c = cross(sub(x4, x2), sub(x3, x2));
        V3<R> d2c = cross(x1x3, x1x4);
        V3<R> d3c = cross(x1x4, x1x2);
        V3<R> d4c = cross(x1x2, x1x3);
        R w1 = v1.inv_mass, w2 = v2.inv_mass, w3 = v3.inv_mass, w4 = v4.inv_mass;
        R denom = w1 * len_sq(d1c) + w2 * len_sq(d2c) + w3 * len_sq(d3c) + w4 * len_sq(d4c) + compliance * inv_dt_sq;
        if (denom < R(1.0e-12f)) return;
        R ml = cval / denom;
        v1.pos = sub(x1, mul(ml * w1, d1c));
        v2.pos = sub(x2, mul(ml * w2, d2c));
        v3.pos = sub(x3, mul(ml * w3, d3c));
        v4.pos = sub(x4, mul(ml * w4, d4c));
    }

    void apply_edge(Body<R> &b, const Edge &c, R compliance, R inv_dt_sq) {  // :573-601
        Vertex<R> &v0 = b.v[c.v[0]], &v1 = b.v[c.v[1]];
        V3<R> x0 = v0.pos, x1 = v1.pos;
        V3<R> delta = sub(x1, x0);
        R length = len(delta);
        R denom = length * (v0.inv_mass + v1.inv_mass + compliance * inv_dt_sq);
        if (denom < R(1.0e-12f)) return;
        V3<R> corr = divs(mul(delta, length - R(c.rest)), denom);
        v0.pos = add(x0, mul(v0.inv_mass, corr));
        v1.pos = sub(x1, mul(v1.inv_mass, corr));
    }

    void apply_lra(Body<R> &b, const LRA &c) {  // :679-698
        const Vertex<R> &v0 = b.v[c.v[0]];
        Vertex<R> &v1 = b.v[c.v[1]];
        V3<R> x0 = v0.pos;
        V3<R> delta = sub(v1.pos, x0);
        R dls = len_sq(delta);
        R md = R(c.max_distance);
        if (dls > md * md) v1.pos = add(x0, divs(mul(delta, md), std::sqrt(dls)));
    }

    void collide_and_update_velocities(Body<R> &b, std::vector<CollidingShape<R>> &shapes, V3<R> g, R dt, uint8_t *flags) {  // :700-825
        R restitution_threshold = R(-2.0f) * len(g) * dt;
        R radius = R(b.cs.vertex_radius);
        bool dynamic = false;
        for (const auto &cs : shapes) dynamic = dynamic || cs.dynamic;
        if (dynamic) {  // dynamic shapes carry velocities from one vertex to the next: in index order
            for (size_t i = 0; i < b.v.size(); ++i) collide_vertex(b.v[i], shapes, dt, restitution_threshold, radius, flags ? flags + i : nullptr);
            return;
        }
        for_vertex_ranges(b.v.size(), [&](size_t first, size_t last) {
            for (size_t i = first; i < last; ++i) collide_vertex(b.v[i], shapes, dt, restitution_threshold, radius, flags ? flags + i : nullptr);
        });
    }

    // one vertex of ApplyCollisionConstraintsAndUpdateVelocities
    void collide_vertex(Vertex<R> &v, std::vector<CollidingShape<R>> &shapes, R dt, R restitution_threshold, R radius, uint8_t *flags) {
        {
            if (!(v.inv_mass > R(0))) return;
            V3<R> prev_v = v.vel;
            v.vel = divs(sub(v.pos, v.prev), dt);
            if (v.shape_idx < 0) return;
            R projected = -(dot(v.pos, v.plane_n) + v.plane_c) + radius;
            const bool replay = flags && freeze_mode == 2;
            const bool contact = replay ? (*flags & 1) != 0 : projected > R(0);
            if (flags && !replay && contact) *flags |= 1;
            if (!contact) return;
            v.contact = true;
            CollidingShape<R> &cs = shapes[v.shape_idx];
            V3<R> n = v.plane_n;
            v.pos = add(v.pos, mul(n, projected));
            if (cs.dynamic) {
                collide_dynamic(v, cs, n, projected, prev_v, dt, restitution_threshold);
                return;
            }
            if (!(cs.isc > R(0))) return;
            // static or kinematic body (:798-816)
            V3<R> v_normal = mul(n, dot(n, v.vel));
            V3<R> v_tan = sub(v.vel, v_normal);
            R vtl = len(v_tan);
            if (vtl > R(0)) {
                R f = cs.friction * projected / (vtl * dt);
                const bool clamped = replay ? (*flags & 2) != 0 : !(f < R(1));  // min(f, 1)
                if (flags && !replay && clamped) *flags |= 2;
                if (clamped) f = R(1);
                v.vel = sub(v.vel, mul(v_tan, f));
            }
            v.vel = sub(v.vel, v_normal);
            R pvn = dot(prev_v, n);
            const bool bounce = replay ? (*flags & 4) != 0 : pvn < restitution_threshold;
            if (flags && !replay && bounce) *flags |= 4;
            if (bounce) v.vel = sub(v.vel, mul(cs.restitution * pvn, n));
        }
    }

    // the dynamic-body branch (:752-797) after the push out of the plane
    static void collide_dynamic(Vertex<R> &v, CollidingShape<R> &cs, V3<R> n, R projected, V3<R> prev_v, R dt, R restitution_threshold) {
        const V3<R> r2 = sub(v.pos, cs.com);
        const V3<R> v2 = add(cs.lin, cross(cs.ang, r2));
        const V3<R> relative = sub(v.vel, v2);
        const V3<R> v_normal = mul(n, dot(n, relative));
        const V3<R> v_tan = sub(relative, v_normal);
        const R vtl = len(v_tan);
        const R vertex_inv_mass = cs.isc * v.inv_mass;
        const V3<R> r2xn = cross(r2, n);
        const R w2 = cs.inv_mass + dot(r2xn, mat4(cs.inertia, cs.inertia[3], r2xn));
        const R w12 = vertex_inv_mass + w2;
        if (!(w12 > R(0))) return;
        V3<R> dv = {R(0), R(0), R(0)};
        if (vtl > R(0)) {
            R f = cs.friction * projected / (vtl * dt);
            if (!(f < R(1))) f = R(1);
            dv = mul(v_tan, f);
        }
        dv = add(dv, v_normal);
        const R pvn = dot(sub(prev_v, v2), n);
        if (pvn < restitution_threshold) dv = add(dv, mul(cs.restitution * pvn, n));
        const V3<R> imp = divs(dv, w12);
        v.vel = sub(v.vel, mul(imp, vertex_inv_mass));
        cs.lin = add(cs.lin, mul(imp, cs.inv_mass));
        cs.ang = add(cs.ang, mat4(cs.inertia, cs.inertia[3], cross(r2, imp)));
        cs.updated = true;
    }

    void update_state(Body<R> &b, R dt, V3<R> disp_g, typename Body<R>::Decisions *dec) {  // :827-921
        if (record_manifold) {  // SoftBodyManifold as OnSoftBodyContactAdded sees it (:832-845, SoftBodyManifold.h)
            b.manifold.assign(b.v.size(), {});
            for (size_t vi = 0; vi < b.v.size(); ++vi) {
                const Vertex<R> &v = b.v[vi];
                std::array<float, 8> &m = b.manifold[vi];
                m[7] = -1.0f;
                if (!v.contact) continue;
                const V3<R> pt = sub(v.pos, mul(v.plane_n, dot(v.pos, v.plane_n) + v.plane_c));
                const V3<R> nrm = neg(v.plane_n);
                m = {1.0f, float(pt.x), float(pt.y), float(pt.z), float(nrm.x), float(nrm.y), float(nrm.z), float(v.shape_idx)};
            }
        }
        R max_sq = R(b.cs.max_linear_velocity) * R(b.cs.max_linear_velocity);
        R max_v_sq = R(0);
        V3<R> lin = {R(0), R(0), R(0)}, ang = {R(0), R(0), R(0)};
        const R big = R(FLT_MAX);
        b.bmin = b.pmin = {big, big, big};
        b.bmax = b.pmax = {-big, -big, -big};
        for (size_t vi = 0; vi < b.v.size(); ++vi) {
            Vertex<R> &v = b.v[vi];
            R vsq = len_sq(v.vel);
            max_v_sq = std::max(max_v_sq, vsq);
            bool clamp = vsq > max_sq;
            if (dec) {
                if (freeze_mode == 2)
                    clamp = dec->vclamp[vi] != 0;
                else
                    dec->vclamp[vi] = clamp ? 1 : 0;
            }
            if (clamp) v.vel = mul(v.vel, std::sqrt(max_sq / vsq));
            lin = add(lin, v.vel);
            ang = add(ang, cross(v.pos, v.vel));
            b.bmin = vmin(b.bmin, v.pos);
            b.bmax = vmax(b.bmax, v.pos);
            V3<R> pred = add(add(v.pos, mul(v.vel, dt)), disp_g);
            b.pmin = vmin(b.pmin, pred);
            b.pmax = vmax(b.pmax, pred);
            reset_collision(v);
        }
        R nvd = R(float(b.v.size() > 0 ? b.v.size() : 1));
        b.lin_vel = divs(lin, nvd);
        b.ang_vel = divs(ang, nvd);
        if (b.cs.update_position) {
            V3<R> delta = mul(R(0.5f), add(b.bmin, b.bmax));
            for (auto &v : b.v) v.pos = sub(v.pos, delta);
            for (auto &p : b.skin_pos) p = sub(p, delta);  // (:889-892)
            b.bmin = sub(b.bmin, delta);
            b.bmax = sub(b.bmax, delta);
            b.pmin = sub(b.pmin, delta);
            b.pmax = sub(b.pmax, delta);
            V3<R> wd;  // Multiply3x3 with identity
            wd.x = (R(1) * delta.x + R(0) * delta.y) + R(0) * delta.z;
            wd.y = (R(0) * delta.x + R(1) * delta.y) + R(0) * delta.z;
            wd.z = (R(0) * delta.x + R(0) * delta.y) + R(1) * delta.z;
            b.position = add(b.position, wd);
        }
        b.skin_prev_valid = false;  // (:916-917)
        // sleep test (:902-915) and deactivation (PhysicsSystem.cpp:2875-2884, BodyManager.cpp:559-561)
        if (b.cs.allow_sleeping) {
            if (max_v_sq > sleep_velocity_threshold) {
                b.sleep_timer = R(0);
            } else {
                b.sleep_timer = b.sleep_timer + dt;
                if (b.sleep_timer >= time_before_sleep) {
                    b.active = false;
                    b.lin_vel = b.ang_vel = {R(0), R(0), R(0)};
                }
            }
        }
        b.force = {R(0), R(0), R(0)};  // ResetForce (:920)
    }
};

struct Handle {
    int use_double;
    std::vector<HullData> hulls;
    double noise = 0.0;
    uint64_t noise_seed = 0, noise_step = 0;
    World<float> wf;
    World<double> wd;
    std::string err;
};

}  // namespace oracle

using namespace oracle;

extern "C" {

void *oracle_world_create(const float gravity[3], int use_double) {
    Handle *h = new Handle();
    h->use_double = use_double;
    h->wf.hulls = h->wd.hulls = &h->hulls;
    h->wf.gravity = {gravity[0], gravity[1], gravity[2]};
    h->wd.gravity = {double(gravity[0]), double(gravity[1]), double(gravity[2])};
    return h;
}

void oracle_world_destroy(void *w) { delete static_cast<Handle *>(w); }

void oracle_set_threads(void *w, int threads) {
    Handle *h = static_cast<Handle *>(w);
    h->wf.threads = threads;
    h->wd.threads = threads;
}

int oracle_add_collider(void *w, int type, const float pos[3], const float half_extent[3], float radius, float friction,
                        float restitution) {
    Handle *h = static_cast<Handle *>(w);
    Collider c;
    c.type = type;
    for (int k = 0; k < 3; ++k) {
        c.pos[k] = pos[k];
        c.half[k] = half_extent ? half_extent[k] : 0.0f;
    }
    c.radius = radius;
    c.friction = friction;
    c.restitution = restitution;
    h->wf.colliders.push_back(c);
    h->wd.colliders.push_back(c);
    return int(h->wf.colliders.size()) - 1;
}

// creation: num_iterations, linear_damping, max_linear_velocity, restitution, friction, pressure,
// gravity_factor, vertex_radius, update_position, allow_sleeping (the last two as float 0/1)
int oracle_add_body(void *w, const uint8_t *blob, size_t len, const float pos[3], const float creation[10]) {
    Handle *h = static_cast<Handle *>(w);
    auto s = std::make_shared<Settings>();
    if (!parse_settings(blob, len, *s, h->err)) return -1;
    if (s->n_rod_ss || s->n_rod_bt) {
        h->err = "rods are not supported";
        return -1;
    }
    Creation cs;
    cs.num_iterations = uint32_t(creation[0]);
    cs.linear_damping = creation[1];
    cs.max_linear_velocity = creation[2];
    cs.restitution = creation[3];
    cs.friction = creation[4];
    cs.pressure = creation[5];
    cs.gravity_factor = creation[6];
    cs.vertex_radius = creation[7];
    cs.update_position = creation[8] != 0.0f;
    cs.allow_sleeping = creation[9] != 0.0f;
    h->wd.add_body(s, pos, cs);
    return h->wf.add_body(s, pos, cs);
}

// BodyInterface::AddForce (EActivation::Activate): sets the step's force, wakes the body and restarts its
// sleep timer (BodyInterface.cpp:699-713).
int oracle_set_force(void *w, int body, const float f[3]) {
    Handle *h = static_cast<Handle *>(w);
    h->wf.bodies[body].force = {f[0], f[1], f[2]};
    h->wd.bodies[body].force = {double(f[0]), double(f[1]), double(f[2])};
    h->wf.bodies[body].active = h->wd.bodies[body].active = true;
    h->wf.bodies[body].sleep_timer = 0.0f;
    h->wd.bodies[body].sleep_timer = 0.0;
    return 0;
}

int oracle_body_active(void *w, int body) { return static_cast<Handle *>(w)->wf.bodies[body].active ? 1 : 0; }

float oracle_body_sleep_timer(void *w, int body) { return static_cast<Handle *>(w)->wf.bodies[body].sleep_timer; }

int oracle_step(void *w, float dt, int collision_steps) {
    Handle *h = static_cast<Handle *>(w);
    if (h->use_double) {
        h->wd.step(double(dt), collision_steps);
        if (h->noise > 0.0) {  // a conditioning probe: a fixed relative perturbation of the state after every step
            ++h->noise_step;
            for (size_t bi = 0; bi < h->wd.bodies.size(); ++bi)
                for (size_t i = 0; i < h->wd.bodies[bi].v.size(); ++i) {
                    Vertex<double> &v = h->wd.bodies[bi].v[i];
                    double *c[6] = {&v.pos.x, &v.pos.y, &v.pos.z, &v.vel.x, &v.vel.y, &v.vel.z};
                    for (int k = 0; k < 6; ++k) {
                        // splitmix64 of (seed, step, body, vertex, component) -> U(-1, 1)
                        uint64_t z = h->noise_seed + 0x9e3779b97f4a7c15ull * (((h->noise_step * 1024 + bi) * 65536 + i) * 8 + k + 1);
                        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
                        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
                        z ^= z >> 31;
                        const double u = double(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
                        *c[k] += h->noise * std::abs(*c[k]) * u;
                    }
                }
        }
    } else {
        h->wf.step(dt, collision_steps);
    }
    return 0;
}

// Records every step's SoftBodyManifold (oracle_get_contacts).
int oracle_set_contact_readback(void *w, int on) {
    Handle *h = static_cast<Handle *>(w);
    h->wf.record_manifold = h->wd.record_manifold = on != 0;
    return 0;
}

// The last step's manifold of one body: 8 floats per vertex {has contact, contact point xyz, normal xyz,
// shape index}. Returns the vertex count (0 when nothing was recorded).
int oracle_get_contacts(void *w, int body, float *out) {
    Handle *h = static_cast<Handle *>(w);
    const auto &m = h->use_double ? h->wd.bodies[body].manifold : h->wf.bodies[body].manifold;
    for (size_t i = 0; i < m.size(); ++i)
        for (int k = 0; k < 8; ++k) out[8 * i + k] = m[i][k];
    return int(m.size());
}

// After a step with host-determined shapes: bit k = shape k is a sensor shape a vertex penetrated.
int oracle_get_sensor_contacts(void *w, int body, uint32_t *mask) {
    Handle *h = static_cast<Handle *>(w);
    *mask = h->use_double ? h->wd.bodies[body].sensor_hits : h->wf.bodies[body].sensor_hits;
    return 0;
}

// Registers a convex hull (points 3 per point, planes 4 per face, face vertex counts and indices);
// returns its index for TableShapeIn::hull.
int oracle_add_hull(void *w, const float *points, int num_points, const float *planes, int num_faces, const uint32_t *counts,
                    const uint32_t *indices) {
    Handle *h = static_cast<Handle *>(w);
    HullData d;
    d.points.assign(points, points + 3 * num_points);
    d.planes.assign(planes, planes + 4 * num_faces);
    size_t next = 0;
    for (int f = 0; f < num_faces; ++f) {
        d.faces.emplace_back(indices + next, indices + next + counts[f]);
        next += counts[f];
    }
    h->hulls.push_back(std::move(d));
    return int(h->hulls.size() - 1);
}

// Host-determined colliding shapes of one body (jsb_colliding_shape layout), used by the following steps
// instead of the world's colliders; n < 0 returns the body to the world's colliders.
int oracle_set_colliding_shapes(void *w, int body, const void *entries, int n) {
    Handle *h = static_cast<Handle *>(w);
    const TableShapeIn *e = static_cast<const TableShapeIn *>(entries);
    for (auto *bs : {&h->wf.bodies[body].table, &h->wd.bodies[body].table}) bs->assign(e, e + (n > 0 ? n : 0));
    h->wf.bodies[body].has_table = h->wd.bodies[body].has_table = n >= 0;
    return 0;
}

// After a step with host-determined shapes: per shape {updated, linear velocity[3], angular velocity[3]}.
// Returns the number of shapes.
int oracle_get_shape_velocities(void *w, int body, float *out) {
    Handle *h = static_cast<Handle *>(w);
    const auto &o = h->use_double ? h->wd.bodies[body].table_out : h->wf.bodies[body].table_out;
    for (size_t k = 0; k < o.size(); ++k)
        for (int j = 0; j < 7; ++j) out[7 * k + j] = o[k][j];
    return int(o.size());
}

// Conditioning probe of double runs: after every step each position and velocity component x becomes
// x (1 + relative u) with u ~ U(-1, 1) fixed by (seed, step, body, vertex, component).
int oracle_set_noise(void *w, double relative, uint64_t seed) {
    Handle *h = static_cast<Handle *>(w);
    h->noise = relative;
    h->noise_seed = seed;
    h->noise_step = 0;
    return 0;
}

int oracle_num_vertices(void *w, int body) { return int(static_cast<Handle *>(w)->wf.bodies[body].v.size()); }

// Writes body position (3), local positions (3N), velocities (3N) as float (double results rounded).
int oracle_get_body(void *w, int body, float *position, float *local_pos, float *vel) {
    Handle *h = static_cast<Handle *>(w);
    auto emit = [&](auto &b) {
        position[0] = float(b.position.x);
        position[1] = float(b.position.y);
        position[2] = float(b.position.z);
        for (size_t i = 0; i < b.v.size(); ++i) {
            local_pos[3 * i + 0] = float(b.v[i].pos.x);
            local_pos[3 * i + 1] = float(b.v[i].pos.y);
            local_pos[3 * i + 2] = float(b.v[i].pos.z);
            if (vel) {
                vel[3 * i + 0] = float(b.v[i].vel.x);
                vel[3 * i + 1] = float(b.v[i].vel.y);
                vel[3 * i + 2] = float(b.v[i].vel.z);
            }
        }
    };
    if (h->use_double)
        emit(h->wd.bodies[body]);
    else
        emit(h->wf.bodies[body]);
    return 0;
}

// World-space positions in double (body position + local), for error reports against FP64.
int oracle_get_world_positions_f64(void *w, int body, double *out) {
    Handle *h = static_cast<Handle *>(w);
    auto emit = [&](auto &b) {
        for (size_t i = 0; i < b.v.size(); ++i) {
            out[3 * i + 0] = double(b.position.x) + double(b.v[i].pos.x);
            out[3 * i + 1] = double(b.position.y) + double(b.v[i].pos.y);
            out[3 * i + 2] = double(b.position.z) + double(b.v[i].pos.z);
        }
    };
    if (h->use_double)
        emit(h->wd.bodies[body]);
    else
        emit(h->wf.bodies[body]);
    return 0;
}

const char *oracle_last_error(void *w) { return static_cast<Handle *>(w)->err.c_str(); }

// FP64 parameter setters for central finite differences (double world only): initial local positions
// and velocities (3 doubles per vertex, may be NULL), per-constraint compliance, force.
// Overwrites the local positions and velocities of a body of the float world (3 floats per vertex each,
// either may be NULL).
int oracle_set_state(void *w, int body, const float *pos3, const float *vel3) {
    Handle *h = static_cast<Handle *>(w);
    auto &b = h->wf.bodies[body];
    for (size_t i = 0; i < b.v.size(); ++i) {
        if (pos3) b.v[i].pos = b.v[i].prev = {pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]};
        if (vel3) b.v[i].vel = {vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2]};
    }
    return 0;
}

int oracle_set_state_f64(void *w, int body, const double *pos3, const double *vel3) {
    Handle *h = static_cast<Handle *>(w);
    auto &b = h->wd.bodies[body];
    for (size_t i = 0; i < b.v.size(); ++i) {
        if (pos3) b.v[i].pos = b.v[i].prev = {pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]};
        if (vel3) b.v[i].vel = {vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2]};
    }
    return 0;
}

int oracle_set_compliance_f64(void *w, int body, const double *edge, int num_edges, const double *vol, int num_vol) {
    Handle *h = static_cast<Handle *>(w);
    auto &b = h->wd.bodies[body];
    if (edge)
        for (int i = 0; i < num_edges && i < int(b.edge_c.size()); ++i) b.edge_c[i] = edge[i];
    if (vol)
        for (int i = 0; i < num_vol && i < int(b.vol_c.size()); ++i) b.vol_c[i] = vol[i];
    return 0;
}

int oracle_set_force_f64(void *w, int body, const double f[3]) {
    Handle *h = static_cast<Handle *>(w);
    h->wd.bodies[body].force = {f[0], f[1], f[2]};
    h->wd.bodies[body].active = true;
    h->wd.bodies[body].sleep_timer = 0.0;
    return 0;
}

// Frozen-decision runs (see World::freeze_mode): 0 off, 1 record, 2 replay.
int oracle_set_freeze(void *w, int mode) {
    Handle *h = static_cast<Handle *>(w);
    h->wf.freeze_mode = h->wd.freeze_mode = mode;
    return 0;
}

// Copies every body's recorded decisions from world src to world dst (same scene) and rewinds them.
// The decisions of a float run, widened to double (a double run that replays a float run's collision
// decisions and planes).
static Body<double>::Decisions widen(const Body<float>::Decisions &f) {
    Body<double>::Decisions d;
    d.shape_collider = f.shape_collider;
    d.shape_friction.assign(f.shape_friction.begin(), f.shape_friction.end());
    d.shape_restitution.assign(f.shape_restitution.begin(), f.shape_restitution.end());
    d.vertex_shape = f.vertex_shape;
    for (const V3<float> &n : f.vertex_n) d.vertex_n.push_back({double(n.x), double(n.y), double(n.z)});
    d.vertex_c.assign(f.vertex_c.begin(), f.vertex_c.end());
    d.flags = f.flags;
    d.vclamp = f.vclamp;
    return d;
}

// Copies the recorded decisions of `src` into `dst` for replay. A float oracle's (use_double = 0)
// decisions also become the double world's, widened.
int oracle_copy_decisions(void *dst, const void *src) {
    Handle *d = static_cast<Handle *>(dst);
    const Handle *s = static_cast<const Handle *>(src);
    if (d->wd.bodies.size() != s->wd.bodies.size()) return -1;
    for (size_t i = 0; i < d->wd.bodies.size(); ++i) {
        if (s->use_double) {
            d->wd.bodies[i].decisions = s->wd.bodies[i].decisions;
        } else {
            d->wd.bodies[i].decisions.clear();
            for (const auto &f : s->wf.bodies[i].decisions) d->wd.bodies[i].decisions.push_back(widen(f));
        }
        d->wd.bodies[i].decision_step = 0;
        d->wf.bodies[i].decisions = s->wf.bodies[i].decisions;
        d->wf.bodies[i].decision_step = 0;
    }
    return 0;
}

// SkinVertices of one body (joint matrices: 16 floats each, Mat44 columns).
int oracle_skin_vertices(void *w, int body, const float *joints, int num_joints, int hard_skin_all) {
    Handle *h = static_cast<Handle *>(w);
    if (h->wf.bodies[body].skin_pos.empty()) return -1;
    h->wf.skin_vertices(h->wf.bodies[body], joints, uint32_t(num_joints), hard_skin_all != 0);
    h->wd.skin_vertices(h->wd.bodies[body], joints, uint32_t(num_joints), hard_skin_all != 0);
    return 0;
}

// SetEnableSkinConstraints / SetSkinnedMaxDistanceMultiplier.
int oracle_set_skin_settings(void *w, int body, int enable, float multiplier) {
    Handle *h = static_cast<Handle *>(w);
    h->wf.bodies[body].skin_enabled = h->wd.bodies[body].skin_enabled = enable != 0;
    h->wf.bodies[body].skin_mult = multiplier;
    h->wd.bodies[body].skin_mult = double(multiplier);
    return 0;
}

// The body's skin states: 9 floats per vertex {previous position, position, normal}; returns the vertex
// count (0 without skinned constraints).
int oracle_get_skin_state(void *w, int body, float *out) {
    Handle *h = static_cast<Handle *>(w);
    if (h->use_double) {
        const auto &b = h->wd.bodies[body];
        for (size_t i = 0; i < b.skin_pos.size(); ++i) {
            const V3<double> *a[3] = {&b.skin_prev[i], &b.skin_pos[i], &b.skin_normal[i]};
            for (int k = 0; k < 3; ++k) {
                out[9 * i + 3 * k] = float(a[k]->x);
                out[9 * i + 3 * k + 1] = float(a[k]->y);
                out[9 * i + 3 * k + 2] = float(a[k]->z);
            }
        }
        return int(b.skin_pos.size());
    }
    const auto &b = h->wf.bodies[body];
    for (size_t i = 0; i < b.skin_pos.size(); ++i) {
        const V3<float> *a[3] = {&b.skin_prev[i], &b.skin_pos[i], &b.skin_normal[i]};
        for (int k = 0; k < 3; ++k) {
            out[9 * i + 3 * k] = a[k]->x;
            out[9 * i + 3 * k + 1] = a[k]->y;
            out[9 * i + 3 * k + 2] = a[k]->z;
        }
    }
    return int(b.skin_pos.size());
}

int oracle_set_sleep_settings(void *w, float time_before_sleep, float point_velocity_sleep_threshold) {
    Handle *h = static_cast<Handle *>(w);
    h->wf.time_before_sleep = time_before_sleep;
    h->wf.sleep_velocity_threshold = point_velocity_sleep_threshold;
    h->wd.time_before_sleep = time_before_sleep;
    h->wd.sleep_velocity_threshold = point_velocity_sleep_threshold;
    return 0;
}

int oracle_get_world_f64(void *w, int body, double *out) {
    Handle *h = static_cast<Handle *>(w);
    auto &b = h->wd.bodies[body];
    for (size_t i = 0; i < b.v.size(); ++i) {
        out[3 * i + 0] = b.position.x + b.v[i].pos.x;
        out[3 * i + 1] = b.position.y + b.v[i].pos.y;
        out[3 * i + 2] = b.position.z + b.v[i].pos.z;
    }
    return 0;
}

}  // extern "C"
