// Host-side mirror of Jolt's SoftBodySharedSettings (Jolt/Physics/SoftBody/SoftBodySharedSettings.h).
//
// TEST AND BENCHMARK INFRASTRUCTURE, not part of the product library (libjsb.so never links it).
// Jolt users keep building their settings with Jolt and hand the GPU the bytes of
// SoftBodySharedSettings::SaveBinaryState. This mirror exists so that the same settings can be
// produced where Jolt is not linked (the GPU test and benchmark hosts): it restates
// CreateConstraints, CalculateEdgeLengths, CalculateLRALengths, CalculateBendConstraintConstants,
// CalculateVolumeConstraintVolumes and Optimize with the same algorithms, tie-breaking and float
// operation order, and writes the same SaveBinaryState byte layout. Its output is compared byte
// for byte with Jolt's in the tests.
#pragma once

#include <cfloat>
#include <cstdint>
#include <string>
#include <vector>

#include "scene_spec.h"

namespace jsb {
namespace host {

class SoftBodySharedSettings {
public:
    using EBendType = scene::BendType;
    using ELRAType = scene::LRAType;
    using VertexAttributes = scene::VertexAttributes;

    struct Vertex {  // 28 bytes, SoftBodySharedSettings.h:127-139
        float mPosition[3] = {0, 0, 0};
        float mVelocity[3] = {0, 0, 0};
        float mInvMass = 1.0f;
    };
    struct Face {  // 16 bytes
        uint32_t mVertex[3];
        uint32_t mMaterialIndex = 0;
    };
    struct Edge {  // 16 bytes
        uint32_t mVertex[2];
        float mRestLength = 1.0f;
        float mCompliance = 0.0f;
        uint32_t GetMinVertexIndex() const { return mVertex[0] < mVertex[1] ? mVertex[0] : mVertex[1]; }
    };
    struct DihedralBend {  // 24 bytes
        uint32_t mVertex[4];
        float mCompliance = 0.0f;
        float mInitialAngle = 0.0f;
        uint32_t GetMinVertexIndex() const;
    };
    struct Volume {  // 24 bytes
        uint32_t mVertex[4];
        float mSixRestVolume = 1.0f;
        float mCompliance = 0.0f;
        uint32_t GetMinVertexIndex() const;
    };
    struct LRA {  // 12 bytes
        uint32_t mVertex[2];
        float mMaxDistance = 0.0f;
        uint32_t GetMinVertexIndex() const { return mVertex[0] < mVertex[1] ? mVertex[0] : mVertex[1]; }
    };
    struct UpdateGroup {  // 28 bytes, SoftBodySharedSettings.h:374-383
        uint32_t mEdgeEndIndex, mLRAEndIndex, mRodStretchShearEndIndex, mRodBendTwistEndIndex, mDihedralBendEndIndex,
            mVolumeEndIndex, mSkinnedEndIndex;
    };

    void CreateConstraints(const VertexAttributes *inVertexAttributes, uint32_t inVertexAttributesLength,
                           EBendType inBendType = EBendType::Distance, float inAngleTolerance = 8.0f * (3.14159265358979323846f / 180.0f));
    void CalculateEdgeLengths();
    void CalculateLRALengths(float inMaxDistanceMultiplier = 1.0f);
    void CalculateBendConstraintConstants();
    void CalculateVolumeConstraintVolumes();
    void Optimize();

    // SaveBinaryState byte layout (SoftBodySharedSettings.cpp:1203-1236); skinned constraints,
    // rods and inverse bind matrices are always written empty by this mirror.
    std::string SaveBinaryState() const;

    std::vector<Vertex> mVertices;
    std::vector<Face> mFaces;
    std::vector<Edge> mEdgeConstraints;
    std::vector<DihedralBend> mDihedralBendConstraints;
    std::vector<Volume> mVolumeConstraints;
    std::vector<LRA> mLRAConstraints;
    std::vector<UpdateGroup> mUpdateGroups;

private:
    struct ClosestKinematic {
        uint32_t mVertex = 0xffffffff;
        uint32_t mHops = 0xffffffff;
        float mDistance = FLT_MAX;
    };
    void CalculateClosestKinematic();
    std::vector<ClosestKinematic> mClosestKinematic;
};

// Builds the settings for one scene body (mesh -> constraints -> Optimize -> optional per-edge
// compliance) exactly like oracle/ref_driver.cpp does with Jolt.
SoftBodySharedSettings build_settings(const scene::MeshSpec &mesh);

}  // namespace host
}  // namespace jsb
