// Matrix.hpp -- row-major 4x4 transform (include/models/Matrix.hpp).
#pragma once

#include "Utils.hpp"

#include <cmath>

template <typename T>
struct Matrix4x4
{
    T values[4][4];

    constexpr Matrix4x4 operator*(const Matrix4x4 &m) const
    {
        Matrix4x4 r{};
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                r.values[i][j] = values[i][0] * m.values[0][j] + values[i][1] * m.values[1][j] +
                                 values[i][2] * m.values[2][j] + values[i][3] * m.values[3][j];
        return r;
    }
    static constexpr Matrix4x4 identity() { return Matrix4x4{{{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}}}; }
    static constexpr Matrix4x4 translation(const Vec3 &o)
    {
        return Matrix4x4{{{1, 0, 0, o.x}, {0, 1, 0, o.y}, {0, 0, 1, o.z}, {0, 0, 0, 1}}};
    }
    // Rotation about a unit axis (Rodrigues' formula).
    static Matrix4x4 rotation(const Vec3 &a, const float angle)
    {
        const float c = std::cos(angle), s = std::sin(angle), t = 1.0f - c;
        return Matrix4x4{{{t * a.x * a.x + c, t * a.x * a.y - s * a.z, t * a.x * a.z + s * a.y, 0},
                          {t * a.x * a.y + s * a.z, t * a.y * a.y + c, t * a.y * a.z - s * a.x, 0},
                          {t * a.x * a.z - s * a.y, t * a.y * a.z + s * a.x, t * a.z * a.z + c, 0},
                          {0, 0, 0, 1}}};
    }
    constexpr Vec3 applyToPosition(const Vec3 &p) const
    {
        return Vec3{values[0][0] * p.x + values[0][1] * p.y + values[0][2] * p.z + values[0][3],
                    values[1][0] * p.x + values[1][1] * p.y + values[1][2] * p.z + values[1][3],
                    values[2][0] * p.x + values[2][1] * p.y + values[2][2] * p.z + values[2][3]};
    }
    constexpr Vec3 applyToDirection(const Vec3 &d) const
    {
        return Vec3{values[0][0] * d.x + values[0][1] * d.y + values[0][2] * d.z,
                    values[1][0] * d.x + values[1][1] * d.y + values[1][2] * d.z,
                    values[2][0] * d.x + values[2][1] * d.y + values[2][2] * d.z};
    }
    constexpr Vec3 getOffset() const { return Vec3{values[0][3], values[1][3], values[2][3]}; }
};

using Matrix4x4f = Matrix4x4<float>;
