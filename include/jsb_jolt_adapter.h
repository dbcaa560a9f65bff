// Jolt-side adapter of the GPU soft-body step (header only; compiles against Jolt Physics and jsb.h).
//
// What a maintainer adds on the Jolt side to run soft bodies on the GPU instead of in
// PhysicsSystem's soft-body jobs (PhysicsSystem.cpp:2701-2897): one GpuSoftBodyStepper per physics system
// and GPU. Settings are uploaded once per SoftBodySharedSettings object, bodies are registered once, and
// each step the stepper
//   1. hands over the forces accumulated on each body (MotionProperties::AddForce),
//   2. determines each body's colliding shapes the way SoftBodyMotionProperties::DetermineCollidingShapes
//      does (SoftBodyMotionProperties.cpp:120-255): a broad-phase query with the body's local bounds U
//      predicted bounds grown by the vertex radius, then for every rigid body that may collide, its convex
//      leaf shapes with their transform relative to the soft body, the combined friction / restitution
//      and, for dynamic bodies, mass, inertia and velocities,
//   3. steps every GPU soft body in one call,
//   4. writes the rigid bodies' velocity changes back (UpdateRigidBodyVelocities, :923-935) and each soft
//      body's state back (SoftBodyMotionProperties::RestoreState, body position).
// Bodies the GPU path does not run (rods, more than 65,536 vertices, a non-identity rotation) are refused
// at AddBody; skinned bodies take their joint matrices through SkinVertices (instead of
// SoftBodyMotionProperties::SkinVertices) and must fit one CTA. With a SoftBodyContactListener set (SetContactListener), every
// candidate body goes through its OnSoftBodyContactValidate like in the reference (rejections, inverse
// mass scales, sensors); without one, sensors are ignored and the default contact settings apply, as in
// the reference. SoftBodyManifold cannot be built outside Jolt (its constructor is private), so the
// contacts OnSoftBodyContactAdded would report reach an adapter callback instead (SetContactCallback):
// per vertex contact flag, local contact point, normal and rigid body, plus the sensors a vertex entered.
// Leaf shapes other than box, sphere, capsule, cylinder and convex hull (meshes, height fields) are not
// collided with: keep bodies that touch them on Jolt's CPU path.
#pragma once

#include <Jolt/Jolt.h>
#include <Jolt/Core/StreamWrapper.h>
#include <Jolt/Physics/PhysicsSystem.h>
#include <Jolt/Physics/StateRecorderImpl.h>
#include <Jolt/Physics/Body/BodyLock.h>
#include <Jolt/Physics/Collision/CollideShape.h>
#include <Jolt/Physics/Collision/CollisionCollectorImpl.h>
#include <Jolt/Physics/Collision/TransformedShape.h>
#include <Jolt/Physics/Collision/Shape/BoxShape.h>
#include <Jolt/Physics/Collision/Shape/CapsuleShape.h>
#include <Jolt/Physics/Collision/Shape/ConvexHullShape.h>
#include <Jolt/Physics/Collision/Shape/CylinderShape.h>
#include <Jolt/Physics/Collision/Shape/SphereShape.h>
#include <Jolt/Physics/SoftBody/SoftBodyContactListener.h>
#include <Jolt/Physics/SoftBody/SoftBodyCreationSettings.h>
#include <Jolt/Physics/SoftBody/SoftBodyMotionProperties.h>

#include <cstring>
#include <functional>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "jsb.h"

namespace jsb_jolt {

// What OnSoftBodyContactAdded's SoftBodyManifold reports for one soft body after a step.
struct SoftBodyContacts {
    JPH::BodyID mSoftBody;
    std::vector<uint8_t> mHasContact;       // per vertex (SoftBodyManifold::HasContact)
    std::vector<float> mLocalContactPoint;  // 3 per vertex (GetLocalContactPoint)
    std::vector<float> mContactNormal;      // 3 per vertex (GetContactNormal)
    std::vector<JPH::BodyID> mContactBody;  // per vertex (GetContactBodyID; invalid without contact)
    std::vector<JPH::BodyID> mSensors;      // GetSensorContactBodyID
};

class GpuSoftBodyStepper {
public:
    explicit GpuSoftBodyStepper(int inDevice) { Check(jsb_context_create(inDevice, &mCtx)); }
    ~GpuSoftBodyStepper() { jsb_context_destroy(mCtx); }
    GpuSoftBodyStepper(const GpuSoftBodyStepper &) = delete;
    GpuSoftBodyStepper &operator=(const GpuSoftBodyStepper &) = delete;

    // After BodyInterface::CreateSoftBody: register the body with the GPU instead of stepping it on the
    // CPU (keep it out of the CPU soft-body jobs, e.g. by a motion flag of your engine).
    bool AddBody(const JPH::BodyID &inID, const JPH::SoftBodyCreationSettings &inCS, JPH::RVec3Arg inPosition) {
        uint32_t settings;
        if (!UploadSettings(inCS.mSettings, settings)) return false;
        jsb_creation_settings c = {};
        c.num_iterations = inCS.mNumIterations;
        c.linear_damping = inCS.mLinearDamping;
        c.max_linear_velocity = inCS.mMaxLinearVelocity;
        c.restitution = inCS.mRestitution;
        c.friction = inCS.mFriction;
        c.pressure = inCS.mPressure;
        c.gravity_factor = inCS.mGravityFactor;
        c.vertex_radius = inCS.mVertexRadius;
        c.update_position = inCS.mUpdatePosition;
        c.make_rotation_identity = inCS.mMakeRotationIdentity;
        c.allow_sleeping = inCS.mAllowSleeping;
        c.faces_double_sided = inCS.mFacesDoubleSided;
        const float p[3] = {float(inPosition.GetX()), float(inPosition.GetY()), float(inPosition.GetZ())};
        uint32_t id;
        if (jsb_body_add(mCtx, settings, &c, p, &id) != JSB_OK) return false;
        mBodies.push_back({inID, id, inCS.mVertexRadius});
        return true;
    }

    // SoftBodyMotionProperties::SkinVertices for a registered body (joint matrices relative to its centre of
    // mass), and its SetEnableSkinConstraints / SetSkinnedMaxDistanceMultiplier; call between steps.
    bool SkinVertices(const JPH::BodyID &inID, const JPH::Mat44 *inJointMatrices, uint32_t inNumJoints, bool inHardSkinAll) {
        const Entry *e = Find(inID);
        if (e == nullptr) return false;
        std::vector<float> m(16 * size_t(inNumJoints));
        for (uint32_t j = 0; j < inNumJoints; ++j)
            for (int c = 0; c < 4; ++c) {
                const JPH::Vec4 col = inJointMatrices[j].GetColumn4(c);
                m[16 * j + 4 * c + 0] = col.GetX();
                m[16 * j + 4 * c + 1] = col.GetY();
                m[16 * j + 4 * c + 2] = col.GetZ();
                m[16 * j + 4 * c + 3] = col.GetW();
            }
        return jsb_body_skin_vertices(mCtx, e->mGpu, m.data(), inNumJoints, inHardSkinAll ? 1 : 0) == JSB_OK;
    }
    bool SetSkinSettings(const JPH::BodyID &inID, bool inEnableSkinConstraints, float inMaxDistanceMultiplier) {
        const Entry *e = Find(inID);
        return e != nullptr && jsb_body_set_skin_settings(mCtx, e->mGpu, inEnableSkinConstraints ? 1 : 0, inMaxDistanceMultiplier) == JSB_OK;
    }

    // The reference's SoftBodyContactListener, consulted for every candidate rigid body (null: none).
    void SetContactListener(JPH::SoftBodyContactListener *inListener) { mListener = inListener; }

    // Called after a step for every soft body that touched a shape or entered a sensor (where the reference
    // calls OnSoftBodyContactAdded); switches the contact readback on.
    void SetContactCallback(std::function<void(const SoftBodyContacts &)> inCallback) {
        mContactCallback = std::move(inCallback);
        Check(jsb_set_contact_readback(mCtx, mContactCallback ? 1 : 0));
    }

    // Replaces the soft-body part of PhysicsSystem::Update for the registered bodies; call it where the
    // soft-body jobs would run (after the rigid bodies' position solve). inStream: the CUDA stream.
    void Step(JPH::PhysicsSystem &ioSystem, float inDeltaTime, int inCollisionSteps, jsb_stream inStream) {
        using namespace JPH;
        const Vec3 g = ioSystem.GetGravity();
        const float gravity[3] = {g.GetX(), g.GetY(), g.GetZ()};
        Check(jsb_set_gravity(mCtx, gravity));
        const BodyLockInterfaceLocking &locks = ioSystem.GetBodyLockInterface();
        mShapes.assign(mBodies.size(), {});
        for (size_t b = 0; b < mBodies.size(); ++b) {
            const Entry &e = mBodies[b];
            {  // MotionProperties::AddForce accumulators, consumed by the step
                BodyLockWrite lock(locks, e.mJolt);
                MotionProperties *mp = lock.GetBody().GetMotionProperties();
                const Vec3 f = mp->GetAccumulatedForce();
                const float force[3] = {f.GetX(), f.GetY(), f.GetZ()};
                Check(jsb_body_add_force(mCtx, e.mGpu, force));
                mp->ResetForce();
            }
            CollectShapes(ioSystem, e, mShapes[b]);
            Check(jsb_body_set_colliding_shapes(mCtx, e.mGpu, mShapes[b].shapes.data(), uint32_t(mShapes[b].shapes.size())));
        }
        Check(jsb_step(mCtx, inDeltaTime, inCollisionSteps, inStream));
        Check(jsb_synchronize(mCtx));
        BodyInterface &bi = ioSystem.GetBodyInterfaceNoLock();
        for (size_t b = 0; b < mBodies.size(); ++b) {
            const Entry &e = mBodies[b];
            WriteBackVelocities(ioSystem, bi, e, mShapes[b]);
            if (mContactCallback) ReportContacts(e, mShapes[b]);
            size_t len = 0;
            Check(jsb_body_save_state(mCtx, e.mGpu, nullptr, 0, &len));
            std::string bytes(len, '\0');
            Check(jsb_body_save_state(mCtx, e.mGpu, &bytes[0], len, &len));
            float p[3];
            Check(jsb_body_read(mCtx, e.mGpu, p, nullptr, nullptr));
            {
                BodyLockWrite lock(ioSystem.GetBodyLockInterfaceNoLock(), e.mJolt);
                StateRecorderImpl rec;
                rec.WriteBytes(bytes.data(), bytes.size());
                rec.Rewind();
                static_cast<SoftBodyMotionProperties *>(lock.GetBody().GetMotionProperties())->RestoreState(rec);
            }
            bi.SetPosition(e.mJolt, RVec3(p[0], p[1], p[2]), EActivation::DontActivate);
        }
    }

private:
    struct Entry {
        JPH::BodyID mJolt;
        uint32_t mGpu;
        float mVertexRadius;
    };
    struct Shapes {  // one soft body's colliding shapes of the current step
        std::vector<jsb_colliding_shape> shapes;
        std::vector<JPH::BodyID> bodies;  // the rigid body of each shape
    };

    const Entry *Find(const JPH::BodyID &inID) const {
        for (const Entry &e : mBodies)
            if (e.mJolt == inID) return &e;
        return nullptr;
    }

    static void PutMatrix(JPH::Mat44Arg inM, float *outColumns, int inColumns) {
        for (int c = 0; c < inColumns; ++c)
            for (int r = 0; r < 3; ++r) outColumns[3 * c + r] = inM(r, c);
    }

    // SoftBodyMotionProperties::DetermineCollidingShapes for one body (:120-255), with the listener's
    // contact settings (or the defaults).
    void CollectShapes(JPH::PhysicsSystem &ioSystem, const Entry &inEntry, Shapes &outShapes) {
        using namespace JPH;
        float lb[6], pb[6];
        Check(jsb_body_bounds(mCtx, inEntry.mGpu, lb, pb));
        AABox local_bounds(Vec3(lb[0], lb[1], lb[2]), Vec3(lb[3], lb[4], lb[5]));
        local_bounds.Encapsulate(AABox(Vec3(pb[0], pb[1], pb[2]), Vec3(pb[3], pb[4], pb[5])));
        local_bounds.ExpandBy(Vec3::sReplicate(inEntry.mVertexRadius));
        const BodyLockInterfaceLocking &locks = ioSystem.GetBodyLockInterface();
        BodyLockRead soft_lock(locks, inEntry.mJolt);
        const Body &soft_body = soft_lock.GetBody();
        const RMat44 com_transform = soft_body.GetCenterOfMassTransform();
        const AABox world_bounds = local_bounds.Transformed(com_transform);
        AllHitCollisionCollector<CollideShapeBodyCollector> hits;
        const ObjectLayer layer = soft_body.GetObjectLayer();
        ioSystem.GetBroadPhaseQuery().CollideAABox(world_bounds, hits, ioSystem.GetDefaultBroadPhaseLayerFilter(layer),
                                                   ioSystem.GetDefaultLayerFilter(layer));
        const RMat44 inverse = com_transform.InversedRotationTranslation();
        for (const BodyID &id : hits.mHits) {
            BodyLockRead lock(ioSystem.GetBodyLockInterfaceNoLock(), id);
            if (!lock.Succeeded()) continue;
            const Body &body = lock.GetBody();
            if (!body.IsRigidBody() || !soft_body.GetCollisionGroup().CanCollide(body.GetCollisionGroup()) ||
                !world_bounds.Overlaps(body.GetWorldSpaceBounds()))
                continue;
            SoftBodyContactSettings settings;
            settings.mIsSensor = body.IsSensor();
            if (mListener == nullptr) {
                if (settings.mIsSensor) continue;  // no listener: sensors are ignored
            } else {
                if (mListener->OnSoftBodyContactValidate(soft_body, body, settings) != SoftBodyValidateResult::AcceptContact) continue;
                if (!settings.mIsSensor && settings.mInvMassScale1 == 0.0f &&
                    (body.GetMotionType() != EMotionType::Dynamic || settings.mInvMassScale2 == 0.0f))
                    continue;  // no interaction
            }
            const Mat44 com = (inverse * body.GetCenterOfMassTransform()).ToMat44();
            jsb_colliding_shape s = {};
            const Shape *shape = body.GetShape();
            switch (shape->GetSubType()) {
                case EShapeSubType::Box: {
                    const Vec3 h = static_cast<const BoxShape *>(shape)->GetHalfExtent();
                    s.type = JSB_COLLIDER_BOX;
                    s.half_extent[0] = h.GetX();
                    s.half_extent[1] = h.GetY();
                    s.half_extent[2] = h.GetZ();
                    break;
                }
                case EShapeSubType::Sphere:
                    s.type = JSB_COLLIDER_SPHERE;
                    s.radius = static_cast<const SphereShape *>(shape)->GetRadius();
                    break;
                case EShapeSubType::Capsule:
                    s.type = JSB_COLLIDER_CAPSULE;
                    s.radius = static_cast<const CapsuleShape *>(shape)->GetRadius();
                    s.half_extent[1] = static_cast<const CapsuleShape *>(shape)->GetHalfHeightOfCylinder();
                    break;
                case EShapeSubType::Cylinder:
                    s.type = JSB_COLLIDER_CYLINDER;
                    s.radius = static_cast<const CylinderShape *>(shape)->GetRadius();
                    s.half_extent[1] = static_cast<const CylinderShape *>(shape)->GetHalfHeight();
                    break;
                case EShapeSubType::ConvexHull:
                    s.type = JSB_COLLIDER_HULL;
                    if (!HullID(static_cast<const ConvexHullShape *>(shape), s.hull_id)) continue;
                    break;
                default:
                    continue;  // not on the GPU path (see the header comment)
            }
            // LeafShape::mTransform as CollectTransformedShapes + the collector rebuild it
            PutMatrix(Mat44::sRotationTranslation(com.GetQuaternion(), com.GetTranslation()), s.transform, 4);
            s.motion_type = settings.mIsSensor ? int32_t(JSB_MOTION_SENSOR) : int32_t(body.GetMotionType());
            s.friction = ioSystem.GetCombineFriction()(soft_body, SubShapeID(), body, SubShapeID());
            s.restitution = ioSystem.GetCombineRestitution()(soft_body, SubShapeID(), body, SubShapeID());
            s.soft_body_inv_mass_scale = settings.mInvMassScale1;
            const Vec3 t = com.GetTranslation();
            s.center_of_mass[0] = t.GetX();
            s.center_of_mass[1] = t.GetY();
            s.center_of_mass[2] = t.GetZ();
            if (!settings.mIsSensor && body.GetMotionType() == EMotionType::Dynamic) {
                const MotionProperties *mp = body.GetMotionProperties();
                s.inv_mass = settings.mInvMassScale2 * mp->GetInverseMass();
                PutMatrix(settings.mInvInertiaScale2 * mp->GetInverseInertiaForRotation(com.GetRotation()), s.inv_inertia, 4);
                const Vec3 lin = inverse.Multiply3x3(mp->GetLinearVelocity()), ang = inverse.Multiply3x3(mp->GetAngularVelocity());
                for (int k = 0; k < 3; ++k) {
                    s.linear_velocity[k] = lin[k];
                    s.angular_velocity[k] = ang[k];
                }
            }
            if (outShapes.shapes.size() == 16) break;  // the GPU keeps 16 shapes per body
            outShapes.shapes.push_back(s);
            outShapes.bodies.push_back(id);
        }
    }

    // UpdateRigidBodyVelocities (:923-935): the soft body's rotation times each dynamic shape's velocity change.
    void WriteBackVelocities(JPH::PhysicsSystem &ioSystem, JPH::BodyInterface &ioBI, const Entry &inEntry, const Shapes &inShapes) {
        using namespace JPH;
        if (inShapes.shapes.empty()) return;
        float out[16 * 7];
        uint32_t n = 0;
        Check(jsb_body_shape_velocities(mCtx, inEntry.mGpu, out, &n));
        RMat44 com_transform;
        {
            BodyLockRead lock(ioSystem.GetBodyLockInterface(), inEntry.mJolt);
            com_transform = lock.GetBody().GetCenterOfMassTransform();
        }
        for (uint32_t k = 0; k < n && k < inShapes.shapes.size(); ++k) {
            const jsb_colliding_shape &s = inShapes.shapes[k];
            if (s.motion_type != JSB_MOTION_DYNAMIC || out[7 * k] == 0.0f) continue;
            const Vec3 lin(out[7 * k + 1], out[7 * k + 2], out[7 * k + 3]), ang(out[7 * k + 4], out[7 * k + 5], out[7 * k + 6]);
            const Vec3 lin0(s.linear_velocity[0], s.linear_velocity[1], s.linear_velocity[2]);
            const Vec3 ang0(s.angular_velocity[0], s.angular_velocity[1], s.angular_velocity[2]);
            ioBI.AddLinearAndAngularVelocity(inShapes.bodies[k], com_transform.Multiply3x3(lin - lin0), com_transform.Multiply3x3(ang - ang0));
        }
    }

    // The step's contacts of one soft body to the contact callback, if it touched a shape or entered a sensor.
    void ReportContacts(const Entry &inEntry, const Shapes &inShapes) {
        uint32_t nv = 0;
        Check(jsb_body_num_vertices(mCtx, inEntry.mGpu, &nv));
        SoftBodyContacts c;
        c.mSoftBody = inEntry.mJolt;
        c.mHasContact.resize(nv);
        c.mLocalContactPoint.resize(3 * size_t(nv));
        c.mContactNormal.resize(3 * size_t(nv));
        std::vector<int32_t> shape(nv);
        Check(jsb_body_contacts(mCtx, inEntry.mGpu, c.mHasContact.data(), c.mLocalContactPoint.data(), c.mContactNormal.data(),
                                shape.data(), nullptr));
        uint32_t sensors = 0;
        Check(jsb_body_sensor_contacts(mCtx, inEntry.mGpu, &sensors));
        bool any = false;
        c.mContactBody.resize(nv);
        for (uint32_t i = 0; i < nv; ++i)
            if (c.mHasContact[i] && shape[i] >= 0 && size_t(shape[i]) < inShapes.bodies.size()) {
                c.mContactBody[i] = inShapes.bodies[size_t(shape[i])];
                any = true;
            }
        for (size_t k = 0; k < inShapes.bodies.size(); ++k)
            if ((sensors >> k) & 1u) {
                bool seen = false;  // a sensor body with several leaf shapes is reported once
                for (const JPH::BodyID &id : c.mSensors) seen = seen || id == inShapes.bodies[k];
                if (!seen) c.mSensors.push_back(inShapes.bodies[k]);
            }
        if (any || !c.mSensors.empty()) mContactCallback(c);
    }

    // Registers a ConvexHullShape once (its points, planes and faces as Jolt built them).
    bool HullID(const JPH::ConvexHullShape *inHull, uint32_t &outID) {
        auto it = mHulls.find(inHull);
        if (it != mHulls.end()) {
            outID = it->second;
            return true;
        }
        std::vector<float> points, planes;
        std::vector<uint32_t> counts, indices;
        for (JPH::uint i = 0; i < inHull->GetNumPoints(); ++i) {
            const JPH::Vec3 p = inHull->GetPoint(i);
            points.insert(points.end(), {p.GetX(), p.GetY(), p.GetZ()});
        }
        JPH::uint face[256];
        for (JPH::uint f = 0; f < inHull->GetNumFaces(); ++f) {
            const JPH::Plane &pl = inHull->GetPlanes()[f];
            planes.insert(planes.end(), {pl.GetNormal().GetX(), pl.GetNormal().GetY(), pl.GetNormal().GetZ(), pl.GetConstant()});
            const JPH::uint n = inHull->GetFaceVertices(f, 256, face);
            counts.push_back(n);
            indices.insert(indices.end(), face, face + n);
        }
        jsb_convex_hull h = {uint32_t(inHull->GetNumPoints()), points.data(), uint32_t(inHull->GetNumFaces()), planes.data(),
                             counts.data(), indices.data()};
        if (jsb_hull_add(mCtx, &h, &outID) != JSB_OK) return false;
        mHulls[inHull] = outID;
        return true;
    }

    bool UploadSettings(const JPH::SoftBodySharedSettings *inSettings, uint32_t &outID) {  // once per settings object
        auto it = mSettings.find(inSettings);
        if (it != mSettings.end()) {
            outID = it->second;
            return true;
        }
        std::stringstream ss;
        JPH::StreamOutWrapper out(ss);
        inSettings->SaveBinaryState(out);  // SoftBodySharedSettings.cpp:1203-1236
        const std::string blob = ss.str();
        if (jsb_settings_upload(mCtx, blob.data(), blob.size(), &outID) != JSB_OK) return false;
        mSettings[inSettings] = outID;
        return true;
    }

    static void Check(jsb_status inStatus) {
        if (inStatus != JSB_OK) JPH_ASSERT(false, jsb_last_error_string());
        (void)inStatus;
    }

    jsb_context *mCtx = nullptr;
    std::unordered_map<const JPH::SoftBodySharedSettings *, uint32_t> mSettings;
    std::unordered_map<const JPH::ConvexHullShape *, uint32_t> mHulls;
    std::vector<Entry> mBodies;
    std::vector<Shapes> mShapes;
    JPH::SoftBodyContactListener *mListener = nullptr;
    std::function<void(const SoftBodyContacts &)> mContactCallback;
};

}  // namespace jsb_jolt
