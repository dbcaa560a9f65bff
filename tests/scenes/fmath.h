// Float3 helpers with the reference's exact operation order (host side).
//
// The soft-body data that the GPU consumes is built on the host (rest lengths, initial dihedral
// angles, rest volumes, LRA lengths, closest-kinematic distances used for sorting). To produce the
// same bytes as Jolt's SoftBodySharedSettings these follow Jolt's Vec3 semantics:
//   dot   = (x*x' + y*y') + (z*z' + 0)    Jolt/Math/Vec3.inl:896-934 (deterministic ReduceSum)
//   cross = separately rounded products   Jolt/Math/Vec3.inl:855-895
//   -v    = 0 - v                         Jolt/Math/Vec3.inl:669-700
// Translation units including this header must be compiled with -ffp-contract=off.
#pragma once

#include <cmath>
#include <cstdint>

namespace jsb {

struct F3 {
    float x, y, z;
};

inline F3 f3(const float *p) { return {p[0], p[1], p[2]}; }
inline F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline F3 operator/(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline F3 neg(F3 a) { return {0.0f - a.x, 0.0f - a.y, 0.0f - a.z}; }
inline float dot(F3 a, F3 b) {
    float px = a.x * b.x, py = a.y * b.y, pz = a.z * b.z;
    return (px + py) + (pz + 0.0f);
}
inline F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length_sq(F3 a) { return dot(a, a); }
inline float length(F3 a) { return std::sqrt(length_sq(a)); }
inline float sign_of(float v) { return v < 0.0f ? -1.0f : 1.0f; }

constexpr float kPi = 3.14159265358979323846f;

// Jolt/Math/Trigonometry.h:48-65
inline float acos_approximate(float x) {
    float ax = std::fabs(x);
    if (ax > 1.0f) ax = 1.0f;
    float val = std::sqrt(1.0f - ax) * (kPi / 2 - 0.175394f * ax);
    return x < 0.0f ? kPi - val : val;
}

}  // namespace jsb
