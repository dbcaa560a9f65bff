// Reference driver: runs the reference's own soft-body solver (Jolt Physics, built from its sources
// by oracle/Makefile.ref) on the seeded scenes of tests/scenes/scene_spec.h and
// dumps what the tests need. TEST INFRASTRUCTURE ONLY: nothing in the product links or runs this.
//
// Bodies are created through the public API only:
//   SoftBodySharedSettings::CreateConstraints / CalculateEdgeLengths / CalculateVolumeConstraintVolumes
//   / Optimize (Jolt/Physics/SoftBody/SoftBodySharedSettings.cpp:189-369, 613-1182),
//   BodyInterface::CreateAndAddSoftBody, PhysicsSystem::Update (Jolt/Physics/PhysicsSystem.cpp:176),
//   SoftBodySharedSettings::SaveBinaryState (SoftBodySharedSettings.cpp:1203-1236),
//   SoftBodyMotionProperties::SaveState (SoftBodyMotionProperties.cpp:1446-1473).
//
// Usage: ref_driver <scene> <out.bin> [key=value ...]
//   scene: pinned_cloth | uneven_batch | large_cloth | diff_cloth | diff_batch
//   keys : steps, dump (comma list of step numbers, 0 = initial), threads, seed, n, n_cloth, n_cube,
//          cloth_min, cloth_max, cube_min, cube_max, time_only (1 = no dumps, print timing JSON)
//
// Scenes with rigid bodies (SceneSpec::rigid) take tables=<path>: for every step, every soft body's
// colliding shapes as the reference determined them (SoftBodyMotionProperties::DetermineCollidingShapes,
// SoftBodyMotionProperties.cpp:120-255), recorded by a SoftBodyContactListener that accepts every contact
// and recomputes the collector's values with the same calls, then each rigid body's velocities after the
// step (which hold the soft bodies' velocity deltas, :923-935):
//   'JSBT' u32 version=4 u32 steps u32 num_rigid
//   per rigid body: u32 num_points, f32[3] per point, u32 num_faces, per face f32[4] plane, u32 count,
//                   count x u32 vertex index (convex hulls; 0, 0 for other shapes)
//   per step: i32 step, u32 num_entries, num_entries x TableEntry, num_rigid x f32[6] (linear, angular
//             velocity after the step, world space), then per soft body u32 n (0 = no contact callback) and
//             n x {u32 has contact, f32[3] local contact point, f32[3] contact normal, i32 rigid index}: the
//             SoftBodyManifold passed to OnSoftBodyContactAdded, then u32 m and m x i32: the rigid indices of
//             its sensor contacts (GetSensorContactBodyID)
// A table entry of a sensor (SoftBodyContactSettings::mIsSensor) has motion 3.
//
// Output file (little endian):
//   'JSBD' u32 version=2 u32 num_dumps u32 scene_len, scene_len bytes of the serialised scene
//          (tests/scenes/scene_io.h, settings bytes written by Jolt)
//   per dump:  i32 step; per body: f32[3] body position, f32[3*N] local positions, f32[3*N] velocities,
//              u32 state_len, state bytes (SaveState)

#include <Jolt/Jolt.h>
#include <Jolt/RegisterTypes.h>
#include <Jolt/Core/Factory.h>
#include <Jolt/Core/TempAllocator.h>
#include <Jolt/Core/JobSystemThreadPool.h>
#include <Jolt/Core/StreamWrapper.h>
#include <Jolt/Physics/PhysicsSettings.h>
#include <Jolt/Physics/PhysicsSystem.h>
#include <Jolt/Physics/StateRecorderImpl.h>
#include <Jolt/Physics/Collision/Shape/BoxShape.h>
#include <Jolt/Physics/Collision/Shape/CapsuleShape.h>
#include <Jolt/Physics/Collision/Shape/ConvexHullShape.h>
#include <Jolt/Physics/Collision/Shape/CylinderShape.h>
#include <Jolt/Physics/Collision/Shape/SphereShape.h>
#include <Jolt/Physics/Body/BodyCreationSettings.h>
#include <Jolt/Physics/SoftBody/SoftBodySharedSettings.h>
#include <Jolt/Physics/SoftBody/SoftBodyCreationSettings.h>
#include <Jolt/Physics/SoftBody/SoftBodyMotionProperties.h>
#include <Jolt/Physics/SoftBody/SoftBodyContactListener.h>
#include <Jolt/Physics/SoftBody/SoftBodyManifold.h>
#include <Jolt/Physics/Body/BodyLockMulti.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>

#include "../tests/scenes/scene_io.h"

using namespace JPH;

namespace {

namespace Layers {
static constexpr ObjectLayer NON_MOVING = 0;
static constexpr ObjectLayer MOVING = 1;
static constexpr ObjectLayer NUM_LAYERS = 2;
}  // namespace Layers

class LayerPairFilter final : public ObjectLayerPairFilter {
public:
    bool ShouldCollide(ObjectLayer a, ObjectLayer b) const override {
        return a == Layers::MOVING || b == Layers::MOVING;
    }
};

class BPLayers final : public BroadPhaseLayerInterface {
public:
    uint GetNumBroadPhaseLayers() const override { return 2; }
    BroadPhaseLayer GetBroadPhaseLayer(ObjectLayer l) const override { return BroadPhaseLayer(BroadPhaseLayer::Type(l)); }
};

class ObjVsBP final : public ObjectVsBroadPhaseLayerFilter {
public:
    bool ShouldCollide(ObjectLayer l, BroadPhaseLayer bp) const override {
        return l == Layers::MOVING || BroadPhaseLayer::Type(bp) == BroadPhaseLayer::Type(Layers::MOVING);
    }
};

SoftBodySharedSettings::VertexAttributes to_jolt(const jsb::scene::VertexAttributes &a) {
    SoftBodySharedSettings::VertexAttributes r;
    r.mCompliance = a.compliance;
    r.mShearCompliance = a.shear_compliance;
    r.mBendCompliance = a.bend_compliance;
    r.mLRAType = SoftBodySharedSettings::ELRAType(int(a.lra_type));
    r.mLRAMaxDistanceMultiplier = a.lra_max_distance_multiplier;
    return r;
}

Ref<SoftBodySharedSettings> build_settings(const jsb::scene::MeshSpec &m) {
    Ref<SoftBodySharedSettings> s = new SoftBodySharedSettings;
    for (size_t i = 0; i < m.positions.size(); ++i) {
        SoftBodySharedSettings::Vertex v;
        v.mPosition = Float3(m.positions[i][0], m.positions[i][1], m.positions[i][2]);
        v.mVelocity = Float3(m.velocities[i][0], m.velocities[i][1], m.velocities[i][2]);
        v.mInvMass = m.inv_mass[i];
        s->mVertices.push_back(v);
    }
    for (auto &f : m.faces) s->AddFace(SoftBodySharedSettings::Face(f[0], f[1], f[2]));
    if (m.create_constraints) {
        SoftBodySharedSettings::VertexAttributes a = to_jolt(m.attributes);
        s->CreateConstraints(&a, 1, SoftBodySharedSettings::EBendType(int(m.bend_type)));
    } else {
        for (size_t i = 0; i < m.edges.size(); ++i)
            s->mEdgeConstraints.push_back(SoftBodySharedSettings::Edge(m.edges[i][0], m.edges[i][1], m.edge_compliance[i]));
        s->CalculateEdgeLengths();
        for (size_t i = 0; i < m.volumes.size(); ++i)
            s->mVolumeConstraints.push_back(SoftBodySharedSettings::Volume(m.volumes[i][0], m.volumes[i][1], m.volumes[i][2],
                                                                          m.volumes[i][3], m.volume_compliance[i]));
        s->CalculateVolumeConstraintVolumes();
    }
    if (!m.skinned.empty()) {  // skinned constraints and inverse bind matrices, then their normals
        for (auto &ib : m.inv_binds) {
            Mat44 mm;
            for (int c = 0; c < 4; ++c)
                mm.SetColumn4(c, Vec4(ib.second[4 * c], ib.second[4 * c + 1], ib.second[4 * c + 2], ib.second[4 * c + 3]));
            s->mInvBindMatrices.push_back(SoftBodySharedSettings::InvBind(ib.first, mm));
        }
        for (auto &k : m.skinned) {
            SoftBodySharedSettings::Skinned sk(k.vertex, k.max_distance, k.backstop_distance, k.backstop_radius);
            for (int w = 0; w < 4; ++w) sk.mWeights[w] = SoftBodySharedSettings::SkinWeight(k.weights[w].first, k.weights[w].second);
            s->mSkinnedConstraints.push_back(sk);
        }
        s->CalculateSkinnedConstraintNormals();
    }
    s->Optimize();
    if (!m.post_optimize_edge_compliance.empty())
        for (size_t i = 0; i < s->mEdgeConstraints.size(); ++i)
            s->mEdgeConstraints[i].mCompliance = m.post_optimize_edge_compliance[i];
    return s;
}

std::string save_settings(const SoftBodySharedSettings &s) {
    std::stringstream ss;
    StreamOutWrapper w(ss);
    s.SaveBinaryState(w);
    return ss.str();
}

void put_u32(FILE *f, uint32_t v) { fwrite(&v, 4, 1, f); }

RefConst<Shape> make_shape(jsb::scene::ColliderType type, const float half_extent[3], float radius) {
    if (type == jsb::scene::ColliderType::Box) return new BoxShape(Vec3(half_extent[0], half_extent[1], half_extent[2]));
    if (type == jsb::scene::ColliderType::Sphere) return new SphereShape(radius);
    if (type == jsb::scene::ColliderType::Capsule) return new CapsuleShape(half_extent[1], radius);
    return new CylinderShape(half_extent[1], radius);
}

// One colliding shape of one soft body in one step (the fields of SoftBodyMotionProperties::CollidingShape
// and its LeafShape), as the tables file stores it.
struct TableEntry {
    uint32_t soft_body, rigid;
    int32_t type, motion;
    float leaf[16];       // LeafShape::mTransform (columns)
    float half_extent[3], radius, friction, restitution;
    float inv_mass_scale1, inv_mass;
    float inv_inertia[16];  // CollidingShape::mInvInertia (columns)
    float com[16];          // CollidingShape::mCenterOfMassTransform (columns)
    float lin[3], ang[3];   // CollidingShape::mLinearVelocity / mAngularVelocity (soft-body space)
    float lin_world[3], ang_world[3];  // the rigid body's velocities when the shape was collected
};

void put_mat(float out[16], Mat44Arg m) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[4 * c + r] = m(r, c);
}

// Accepts every contact and records, per soft body, what SoftBodyMotionProperties::DetermineCollidingShapes'
// collector stores for the shape (SoftBodyMotionProperties.cpp:139-225), computed with the same calls.
class TableRecorder final : public SoftBodyContactListener {
public:
    std::map<uint32_t, uint32_t> soft_index, rigid_index;  // BodyID index -> spec index
    const jsb::scene::SceneSpec *spec = nullptr;
    const PhysicsSystem *system = nullptr;
    std::mutex mutex;
    std::vector<TableEntry> entries;  // of the current step

    SoftBodyValidateResult OnSoftBodyContactValidate(const Body &inSoftBody, const Body &inOtherBody, SoftBodyContactSettings &ioSettings) override {
        TableEntry e{};
        e.soft_body = soft_index.at(inSoftBody.GetID().GetIndex());
        e.rigid = rigid_index.at(inOtherBody.GetID().GetIndex());
        const jsb::scene::RigidSpec &rs = spec->rigid[e.rigid];
        e.type = int32_t(rs.type);
        e.motion = ioSettings.mIsSensor ? 3 : int32_t(inOtherBody.GetMotionType());
        RMat44 inverse = inSoftBody.GetCenterOfMassTransform().InversedRotationTranslation();
        Mat44 com = (inverse * inOtherBody.GetCenterOfMassTransform()).ToMat44();
        put_mat(e.com, com);
        put_mat(e.leaf, Mat44::sRotationTranslation(com.GetQuaternion(), com.GetTranslation()));
        for (int k = 0; k < 3; ++k) e.half_extent[k] = rs.half_extent[k];
        e.radius = rs.radius;
        e.friction = system->GetCombineFriction()(inSoftBody, SubShapeID(), inOtherBody, SubShapeID());
        e.restitution = system->GetCombineRestitution()(inSoftBody, SubShapeID(), inOtherBody, SubShapeID());
        e.inv_mass_scale1 = ioSettings.mInvMassScale1;
        if (inOtherBody.GetMotionType() == EMotionType::Dynamic) {
            const MotionProperties *mp = inOtherBody.GetMotionProperties();
            e.inv_mass = ioSettings.mInvMassScale2 * mp->GetInverseMass();
            put_mat(e.inv_inertia, ioSettings.mInvInertiaScale2 * mp->GetInverseInertiaForRotation(com.GetRotation()));
            Vec3 lin = inverse.Multiply3x3(mp->GetLinearVelocity()), ang = inverse.Multiply3x3(mp->GetAngularVelocity());
            Vec3 lw = mp->GetLinearVelocity(), aw = mp->GetAngularVelocity();
            for (int k = 0; k < 3; ++k) {
                e.lin[k] = lin[k];
                e.ang[k] = ang[k];
                e.lin_world[k] = lw[k];
                e.ang_world[k] = aw[k];
            }
        }
        std::lock_guard<std::mutex> lock(mutex);
        entries.push_back(e);
        return SoftBodyValidateResult::AcceptContact;
    }

    // SoftBodyManifold of each soft body that had a contact this step (SoftBodyMotionProperties.cpp:832-845)
    struct ManifoldVertex {
        uint32_t has;
        float point[3], normal[3];
        int32_t rigid;
    };
    std::map<uint32_t, std::vector<ManifoldVertex>> manifolds;
    std::map<uint32_t, std::vector<int32_t>> sensor_contacts;

    void OnSoftBodyContactAdded(const Body &inSoftBody, const SoftBodyManifold &inManifold) override {
        std::vector<ManifoldVertex> out;
        for (const SoftBodyVertex &v : inManifold.GetVertices()) {
            ManifoldVertex m{};
            m.rigid = -1;
            if (inManifold.HasContact(v)) {
                m.has = 1;
                Vec3 p = inManifold.GetLocalContactPoint(v), n = inManifold.GetContactNormal(v);
                for (int k = 0; k < 3; ++k) {
                    m.point[k] = p[k];
                    m.normal[k] = n[k];
                }
                BodyID id = inManifold.GetContactBodyID(v);
                m.rigid = rigid_index.count(id.GetIndex()) ? int32_t(rigid_index.at(id.GetIndex())) : -2;
            }
            out.push_back(m);
        }
        std::vector<int32_t> sensors;
        for (uint i = 0; i < inManifold.GetNumSensorContacts(); ++i) {
            BodyID id = inManifold.GetSensorContactBodyID(i);
            sensors.push_back(rigid_index.count(id.GetIndex()) ? int32_t(rigid_index.at(id.GetIndex())) : -2);
        }
        std::lock_guard<std::mutex> lock(mutex);
        manifolds[soft_index.at(inSoftBody.GetID().GetIndex())] = std::move(out);
        sensor_contacts[soft_index.at(inSoftBody.GetID().GetIndex())] = std::move(sensors);
    }
};

}  // namespace

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: ref_driver <scene> <out.bin> [key=value ...]\n");
        return 2;
    }
    std::string scene_name = argv[1];
    std::string out_path = argv[2];
    std::map<std::string, std::string> kv;
    for (int i = 3; i < argc; ++i) {
        const char *eq = strchr(argv[i], '=');
        if (!eq) continue;
        kv[std::string(argv[i], eq - argv[i])] = eq + 1;
    }
    auto geti = [&](const char *k, long d) { return kv.count(k) ? std::stol(kv[k]) : d; };

    std::string params;
    for (auto &p : kv) params += p.first + "=" + p.second + " ";
    jsb::scene::SceneSpec spec;
    if (!jsb::scene::make_named_scene(scene_name, params, spec)) {
        fprintf(stderr, "unknown scene %s\n", scene_name.c_str());
        return 2;
    }
    int steps = int(geti("steps", spec.num_steps));
    int threads = int(geti("threads", 1));
    bool time_only = geti("time_only", 0) != 0;
    std::vector<int> dump_steps;
    if (kv.count("dump")) {
        std::stringstream ds(kv["dump"]);
        std::string tok;
        while (std::getline(ds, tok, ',')) dump_steps.push_back(std::stoi(tok));
    } else
        dump_steps = {0, 1, steps};

    RegisterDefaultAllocator();
    Factory::sInstance = new Factory();
    RegisterTypes();
    {
        TempAllocatorImpl temp_allocator(512 * 1024 * 1024);
        JobSystemThreadPool job_system(cMaxPhysicsJobs, cMaxPhysicsBarriers, threads - 1);
        BPLayers bp_layers;
        ObjVsBP obj_vs_bp;
        LayerPairFilter pair_filter;
        PhysicsSystem system;
        system.Init(uint(spec.bodies.size() + spec.colliders.size() + spec.rigid.size() + 16), 0, 65536, 65536, bp_layers, obj_vs_bp,
                    pair_filter);
        system.SetGravity(Vec3(spec.gravity[0], spec.gravity[1], spec.gravity[2]));
        BodyInterface &bi = system.GetBodyInterface();

        for (auto &c : spec.colliders) {
            BodyCreationSettings bcs(make_shape(c.type, c.half_extent, c.radius), RVec3(c.position[0], c.position[1], c.position[2]),
                                     Quat::sIdentity(), EMotionType::Static, Layers::NON_MOVING);
            bcs.mFriction = c.friction;
            bcs.mRestitution = c.restitution;
            bi.CreateAndAddBody(bcs, EActivation::DontActivate);
        }
        TableRecorder recorder;
        recorder.spec = &spec;
        recorder.system = &system;
        std::vector<BodyID> rigid_ids;
        for (size_t r = 0; r < spec.rigid.size(); ++r) {
            const jsb::scene::RigidSpec &c = spec.rigid[r];
            const bool moving = c.motion != 0;
            RefConst<Shape> shape;
            if (c.type == jsb::scene::ColliderType::Hull) {
                Array<Vec3> pts;
                for (auto &q : c.hull_points) pts.push_back(Vec3(q[0], q[1], q[2]));
                shape = ConvexHullShapeSettings(pts).Create().Get();
            } else {
                shape = make_shape(c.type, c.half_extent, c.radius);
            }
            BodyCreationSettings bcs(shape, RVec3(c.position[0], c.position[1], c.position[2]),
                                     Quat(c.rotation[0], c.rotation[1], c.rotation[2], c.rotation[3]), EMotionType(c.motion),
                                     moving ? Layers::MOVING : Layers::NON_MOVING);
            bcs.mFriction = c.friction;
            bcs.mRestitution = c.restitution;
            bcs.mIsSensor = c.sensor;
            if (c.motion == 2) {
                bcs.mOverrideMassProperties = EOverrideMassProperties::CalculateInertia;
                bcs.mMassPropertiesOverride.mMass = c.mass;
            }
            bcs.mLinearVelocity = Vec3(c.velocity[0], c.velocity[1], c.velocity[2]);
            bcs.mAngularVelocity = Vec3(c.angular_velocity[0], c.angular_velocity[1], c.angular_velocity[2]);
            BodyID id = bi.CreateAndAddBody(bcs, moving ? EActivation::Activate : EActivation::DontActivate);
            rigid_ids.push_back(id);
            recorder.rigid_index[id.GetIndex()] = uint32_t(r);
        }

        std::vector<Ref<SoftBodySharedSettings>> settings;
        std::vector<BodyID> ids;
        for (auto &b : spec.bodies) {
            settings.push_back(build_settings(b.mesh));
            SoftBodyCreationSettings sbcs(settings.back(), RVec3(b.position[0], b.position[1], b.position[2]), Quat::sIdentity(),
                                          Layers::MOVING);
            sbcs.mNumIterations = b.creation.num_iterations;
            sbcs.mLinearDamping = b.creation.linear_damping;
            sbcs.mMaxLinearVelocity = b.creation.max_linear_velocity;
            sbcs.mRestitution = b.creation.restitution;
            sbcs.mFriction = b.creation.friction;
            sbcs.mPressure = b.creation.pressure;
            sbcs.mGravityFactor = b.creation.gravity_factor;
            sbcs.mVertexRadius = b.creation.vertex_radius;
            sbcs.mUpdatePosition = b.creation.update_position;
            sbcs.mMakeRotationIdentity = b.creation.make_rotation_identity;
            sbcs.mAllowSleeping = b.creation.allow_sleeping;
            sbcs.mFacesDoubleSided = b.creation.faces_double_sided;
            ids.push_back(bi.CreateAndAddSoftBody(sbcs, EActivation::Activate));
            recorder.soft_index[ids.back().GetIndex()] = uint32_t(ids.size() - 1);
        }
        system.OptimizeBroadPhase();
        // Skinned bodies (skin=<path>): before every step the joints' matrices relative to the body's centre
        // of mass go to SoftBodyMotionProperties::SkinVertices (hard skinning on the first step); the
        // maximum distance multiplier becomes 1.5 from step 40 and skin constraints are off for steps 61-65.
        // Per step and skinned body: i32 step, u32 body, f32 multiplier, u32 enabled, u32 hard, 2 x 16 f32.
        FILE *skin = nullptr;
        if (kv.count("skin")) {
            skin = fopen(kv["skin"].c_str(), "wb");
            if (!skin) {
                fprintf(stderr, "cannot open %s\n", kv["skin"].c_str());
                return 1;
            }
            fwrite("JSBK", 4, 1, skin);
        }
        FILE *tables = nullptr;
        if (!spec.rigid.empty() && kv.count("tables")) {
            system.SetSoftBodyContactListener(&recorder);
            tables = fopen(kv["tables"].c_str(), "wb");
            if (!tables) {
                fprintf(stderr, "cannot open %s\n", kv["tables"].c_str());
                return 1;
            }
            fwrite("JSBT", 4, 1, tables);
            put_u32(tables, 4);
            put_u32(tables, uint32_t(steps));
            put_u32(tables, uint32_t(spec.rigid.size()));
            // per rigid body, its convex hull as ConvexHullShape holds it (points relative to the centre of
            // mass, one plane per face, each face's vertex indices); nothing for other shapes
            BodyLockInterfaceNoLock const &lk = system.GetBodyLockInterfaceNoLock();
            for (BodyID id : rigid_ids) {
                BodyLockRead lock(lk, id);
                const Shape *sh = lock.GetBody().GetShape();
                if (sh->GetSubType() != EShapeSubType::ConvexHull) {
                    put_u32(tables, 0);
                    put_u32(tables, 0);
                    continue;
                }
                const ConvexHullShape *hull = static_cast<const ConvexHullShape *>(sh);
                put_u32(tables, hull->GetNumPoints());
                for (uint i = 0; i < hull->GetNumPoints(); ++i) {
                    Vec3 q = hull->GetPoint(i);
                    float f3[3] = {q.GetX(), q.GetY(), q.GetZ()};
                    fwrite(f3, 4, 3, tables);
                }
                put_u32(tables, hull->GetNumFaces());
                for (uint i = 0; i < hull->GetNumFaces(); ++i) {
                    const Plane &pl = hull->GetPlanes()[i];
                    float f4[4] = {pl.GetNormal().GetX(), pl.GetNormal().GetY(), pl.GetNormal().GetZ(), pl.GetConstant()};
                    fwrite(f4, 4, 4, tables);
                    uint idx[256];
                    const uint nfv = hull->GetFaceVertices(i, 256, idx);
                    put_u32(tables, nfv);
                    for (uint k = 0; k < nfv; ++k) put_u32(tables, idx[k]);
                }
            }
        }

        FILE *f = nullptr;
        if (!time_only) {
            f = fopen(out_path.c_str(), "wb");
            if (!f) {
                fprintf(stderr, "cannot open %s\n", out_path.c_str());
                return 1;
            }
            size_t body_index = 0;
            std::string scene_bytes = jsb::scene::serialize_scene(spec, [&](const jsb::scene::MeshSpec &) {
                return save_settings(*settings[body_index++]);
            });
            fwrite("JSBD", 4, 1, f);
            put_u32(f, 2);
            put_u32(f, uint32_t(dump_steps.size()));
            put_u32(f, uint32_t(scene_bytes.size()));
            fwrite(scene_bytes.data(), 1, scene_bytes.size(), f);
        }
        auto dump = [&](int step) {
            int32_t st = step;
            fwrite(&st, 4, 1, f);
            BodyLockInterfaceNoLock const &lock_if = system.GetBodyLockInterfaceNoLock();
            for (BodyID id : ids) {
                BodyLockRead lock(lock_if, id);
                const Body &body = lock.GetBody();
                RVec3 p = body.GetPosition();
                float pf[3] = {float(p.GetX()), float(p.GetY()), float(p.GetZ())};
                fwrite(pf, 4, 3, f);
                const SoftBodyMotionProperties *mp = static_cast<const SoftBodyMotionProperties *>(body.GetMotionProperties());
                const auto &verts = mp->GetVertices();
                std::vector<float> buf(verts.size() * 3);
                for (size_t i = 0; i < verts.size(); ++i) {
                    buf[3 * i + 0] = verts[i].mPosition.GetX();
                    buf[3 * i + 1] = verts[i].mPosition.GetY();
                    buf[3 * i + 2] = verts[i].mPosition.GetZ();
                }
                fwrite(buf.data(), 4, buf.size(), f);
                for (size_t i = 0; i < verts.size(); ++i) {
                    buf[3 * i + 0] = verts[i].mVelocity.GetX();
                    buf[3 * i + 1] = verts[i].mVelocity.GetY();
                    buf[3 * i + 2] = verts[i].mVelocity.GetZ();
                }
                fwrite(buf.data(), 4, buf.size(), f);
                StateRecorderImpl rec;
                mp->SaveState(rec);
                std::string data = rec.GetData();
                put_u32(f, uint32_t(data.size()));
                fwrite(data.data(), 1, data.size(), f);
            }
        };

        size_t next_dump = 0;
        if (!time_only && next_dump < dump_steps.size() && dump_steps[next_dump] == 0) {
            dump(0);
            ++next_dump;
        }
        uint64_t total_vertices = 0, vi_per_step = 0;
        for (size_t b = 0; b < spec.bodies.size(); ++b) {
            total_vertices += spec.bodies[b].mesh.positions.size();
            vi_per_step += uint64_t(spec.bodies[b].mesh.positions.size()) * spec.bodies[b].creation.num_iterations * spec.collision_steps;
        }
        double seconds = 0.0;
        for (int step = 1; step <= steps; ++step) {
            for (size_t b = 0; b < spec.bodies.size(); ++b) {
                const float *fv = spec.bodies[b].force;
                if (fv[0] != 0.0f || fv[1] != 0.0f || fv[2] != 0.0f) bi.AddForce(ids[b], Vec3(fv[0], fv[1], fv[2]));
            }
            for (size_t b = 0; b < spec.bodies.size() && skin; ++b) {
                if (spec.bodies[b].mesh.skinned.empty()) continue;
                const float phi = 6.2831853f * float(step) / 60.0f;
                const Mat44 j0 = Mat44::sTranslation(Vec3(0.3f * std::sin(phi), 1.5f, 0.0f)) * Mat44::sRotationX(0.2f * std::sin(phi));
                const Mat44 j1 = j0 * Mat44::sTranslation(Vec3(0.0f, 0.0f, 0.6f)) * Mat44::sRotationX(0.3f * std::sin(phi));
                BodyLockWrite lock(system.GetBodyLockInterface(), ids[b]);
                Body &body = lock.GetBody();
                SoftBodyMotionProperties *mp = static_cast<SoftBodyMotionProperties *>(body.GetMotionProperties());
                const RMat44 com = body.GetCenterOfMassTransform();
                const Mat44 inv = com.InversedRotationTranslation().ToMat44();
                const Mat44 joints[2] = {inv * j0, inv * j1};
                const float mult = step >= 40 ? 1.5f : 1.0f;
                const bool enabled = !(step >= 61 && step <= 65);
                const bool hard = step == 1;
                mp->SetSkinnedMaxDistanceMultiplier(mult);
                mp->SetEnableSkinConstraints(enabled);
                mp->SkinVertices(com, joints, 2, hard, temp_allocator);
                int32_t st = step;
                fwrite(&st, 4, 1, skin);
                put_u32(skin, uint32_t(b));
                fwrite(&mult, 4, 1, skin);
                put_u32(skin, enabled ? 1u : 0u);
                put_u32(skin, hard ? 1u : 0u);
                for (const Mat44 &m : joints)
                    for (int c = 0; c < 4; ++c) {
                        const Vec4 col = m.GetColumn4(c);
                        float f4[4] = {col.GetX(), col.GetY(), col.GetZ(), col.GetW()};
                        fwrite(f4, 4, 4, skin);
                    }
            }
            auto t0 = std::chrono::steady_clock::now();
            EPhysicsUpdateError err = system.Update(spec.dt, spec.collision_steps, &temp_allocator, &job_system);
            auto t1 = std::chrono::steady_clock::now();
            seconds += std::chrono::duration<double>(t1 - t0).count();
            if (err != EPhysicsUpdateError::None) {
                fprintf(stderr, "update error %d at step %d\n", int(err), step);
                return 1;
            }
            if (!time_only && next_dump < dump_steps.size() && dump_steps[next_dump] == step) {
                dump(step);
                ++next_dump;
            }
            if (tables) {
                // entries of one soft body keep their collection order; soft bodies in index order
                std::stable_sort(recorder.entries.begin(), recorder.entries.end(),
                                 [](const TableEntry &a, const TableEntry &b) { return a.soft_body < b.soft_body; });
                int32_t st = step;
                fwrite(&st, 4, 1, tables);
                put_u32(tables, uint32_t(recorder.entries.size()));
                fwrite(recorder.entries.data(), sizeof(TableEntry), recorder.entries.size(), tables);
                recorder.entries.clear();
                for (BodyID id : rigid_ids) {
                    Vec3 lv = bi.GetLinearVelocity(id), av = bi.GetAngularVelocity(id);
                    float v6[6] = {lv.GetX(), lv.GetY(), lv.GetZ(), av.GetX(), av.GetY(), av.GetZ()};
                    fwrite(v6, 4, 6, tables);
                }
                for (uint32_t b = 0; b < uint32_t(ids.size()); ++b) {  // manifolds (none: 0)
                    auto it = recorder.manifolds.find(b);
                    put_u32(tables, it == recorder.manifolds.end() ? 0u : uint32_t(it->second.size()));
                    if (it != recorder.manifolds.end())
                        fwrite(it->second.data(), sizeof(TableRecorder::ManifoldVertex), it->second.size(), tables);
                    auto sit = recorder.sensor_contacts.find(b);
                    const uint32_t ns = sit == recorder.sensor_contacts.end() ? 0u : uint32_t(sit->second.size());
                    put_u32(tables, ns);
                    if (ns) fwrite(sit->second.data(), 4, ns, tables);
                }
                recorder.manifolds.clear();
                recorder.sensor_contacts.clear();
            }
        }
        if (f) fclose(f);
        if (tables) fclose(tables);
        if (skin) fclose(skin);
        printf("{\"scene\": \"%s\", \"bodies\": %zu, \"vertices\": %llu, \"steps\": %d, \"threads\": %d, \"seconds\": %.6f, "
               "\"vertex_iterations_per_s\": %.6e}\n",
               scene_name.c_str(), spec.bodies.size(), (unsigned long long)total_vertices, steps, threads, seconds,
               double(vi_per_step) * steps / (seconds > 0 ? seconds : 1e-30));
    }
    UnregisterTypes();
    delete Factory::sInstance;
    Factory::sInstance = nullptr;
    return 0;
}
