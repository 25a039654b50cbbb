// oracle_common.hpp -- FP32 vector helpers of the oracle (TEST INFRASTRUCTURE).
// Each helper evaluates its expression in the same order as the matching
// member of Vec3 in include/Utils.hpp:76-118 (DevilRay), so that with
// -ffp-contract=off the results round identically.
#pragma once

#include <cmath>

namespace oracle {

struct V3 {
    float x, y, z;
};

inline V3 sub(const V3 &a, const V3 &b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(const V3 &a, const V3 &b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mulv(const V3 &a, const V3 &b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 mul(const V3 &a, float f) { return V3{a.x * f, a.y * f, a.z * f}; }
// Vec3::operator/(float) multiplies by the reciprocal (Utils.hpp:86).
inline V3 divs(const V3 &a, float f) { return mul(a, 1.0f / f); }
inline float dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3 &a, const V3 &v)
{
    return V3{a.y * v.z - a.z * v.y, a.z * v.x - a.x * v.z, a.x * v.y - a.y * v.x};
}
inline float length(const V3 &a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// Vec3::normalized (Utils.hpp:94-97) divides each component by the length.
inline V3 normalized(const V3 &a)
{
    const float l = length(a);
    return V3{a.x / l, a.y / l, a.z / l};
}
inline bool anyNan(const V3 &a) { return std::isnan(a.x) || std::isnan(a.y) || std::isnan(a.z); }
inline V3 inv(const V3 &a) { return V3{1 / a.x, 1 / a.y, 1 / a.z}; }

// std::min / std::max as libstdc++ defines them: the first argument wins
// unless the comparison says otherwise (matters for NaN and signed zeros).
inline float stdMin(float a, float b) { return (b < a) ? b : a; }
inline float stdMax(float a, float b) { return (a < b) ? b : a; }

}  // namespace oracle
