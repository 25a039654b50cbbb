// DistributionSamplers.hpp -- sampling helpers and alias tables
// (include/tracing/DistributionSamplers.hpp of the reference). `Rng` is any
// type with `float rnd()` returning a uniform in [0, 1] (or (0, 1]).
#pragma once

#include "device/Array.hpp"
#include "devilray_gb300.h"
#include "Utils.hpp"

#include <cmath>
#include <span>

// Uniform direction: azimuth 2 pi u0, polar angle acos(1 - 2 u1).
template <typename Rng>
Vec3 uniformSphereSample(Rng &r)
{
    const float theta0 = 2 * pi * r.rnd();
    const float theta1 = std::acos(1 - 2 * r.rnd());
    return Vec3{std::sin(theta1) * std::sin(theta0), std::sin(theta1) * std::cos(theta0), std::cos(theta1)};
}

template <typename Rng>
Vec3 uniformHemisphereSample(const Vec3 &normal, Rng &r)
{
    const Vec3 v = uniformSphereSample(r);
    return v.dot(normal) < 0 ? v * -1 : v;
}

// Cosine-weighted direction about `normal`: a uniform sphere point plus the
// normal, normalised.
template <typename Rng>
Vec3 cosineWeightedHemisphereSample(const Vec3 &normal, Rng &r)
{
    return (uniformSphereSample(r) + normal).normalized();
}

// One slot of an alias table; the layout of dr_alias_entry.
struct AliasEntry
{
    float p_A;
    float pdf_A;
    float pdf_B;
    int A;
    int B;
};
static_assert(sizeof(AliasEntry) == sizeof(dr_alias_entry), "AliasEntry must match dr_alias_entry");

struct AliasTable
{
    DeviceArray<AliasEntry> entries;
};

struct AliasSample
{
    int index;
    float pdf;
};

// Draws an index: slot floor(r0 * n) (r0 = 1 maps to the last slot), then A if
// r1 <= p_A, else B.
template <typename Rng>
AliasSample sample(std::span<const AliasEntry> table, Rng &rng)
{
    const float r = rng.rnd();
    float findex = r * table.size();
    if (findex == table.size()) findex = table.size() - 1;
    const int index = static_cast<int>(findex);
    const float p = rng.rnd();
    const AliasEntry &e = table[index];
    if (p <= e.p_A) return AliasSample{e.A, e.pdf_A};
    return AliasSample{e.B, e.pdf_B};
}

// The alias table of generateAliasTable (src/DistributionSamplers.cpp:39-149),
// built on the device by dr_alias_build (bit-identical table). Negative
// weights count as 0; a total below 1e-5 gives the uniform table.
AliasTable generateAliasTable(std::span<const float> importances);

// Uniform point on triangle ABC from two uniforms (reflected when u + v > 1).
template <typename Rng>
Vec3 uniformTriangleSample(const Vec3 &A, const Vec3 &B, const Vec3 &C, Rng &rng)
{
    float u = rng.rnd();
    float v = rng.rnd();
    if (u + v > 1) {
        u = 1 - u;
        v = 1 - v;
    }
    return A + (B - A) * u + (C - A) * v;
}
