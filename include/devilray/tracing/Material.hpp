// Material.hpp -- the two material kinds of the reference
// (include/tracing/Material.hpp): a dielectric with an inside medium, or a
// diffuse surface with emission and reflectance. A Renderer converts them to
// dr_material records.
#pragma once

#include "Utils.hpp"
#include "tracing/Medium.hpp"

#include <variant>

struct BaseMaterial
{
    Vec4 debug_color;
};

struct TransparentMaterial : BaseMaterial
{
    Medium inside_medium;
};

struct DiffuseMaterial : BaseMaterial
{
    Vec4 emission;
    Vec4 diffuse_reflectance;
};

using Material = std::variant<TransparentMaterial, DiffuseMaterial>;

inline Vec4 getDebugColor(const Material &mat)
{
    return std::visit([](const auto &m) { return m.debug_color; }, mat);
}

// Emitted radiant exitance: pi x emission for a diffuse emitter, none for a
// dielectric (include/tracing/LightSampling.hpp:7-13).
inline Vec4 radiantExitance(const Material &mat)
{
    if (const auto *d = std::get_if<DiffuseMaterial>(&mat)) return d->emission * pi;
    return Vec4{0, 0, 0, 0};
}
