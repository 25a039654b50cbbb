// Utils.hpp -- value types of the DevilRay host interface (include/Utils.hpp of
// the reference): vectors, sizes, rays, boxes and the small colour and
// geometry helpers that scene-building code uses. Host-only: the device side
// of this library is behind the C ABI of devilray_gb300.h.
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <limits>
#include <numbers>
#include <ostream>

#ifndef HD
#define HD
#endif

struct Timer
{
    Timer() : start_time(std::chrono::steady_clock::now()) {}
    float elapsedSeconds() const
    {
        return std::chrono::duration<float>(std::chrono::steady_clock::now() - start_time).count();
    }

private:
    std::chrono::steady_clock::time_point start_time;
};

constexpr float pi = std::numbers::pi_v<float>;

struct ColorRGBA8
{
    uint8_t r, g, b, a;
};

struct Vec4
{
    float x, y, z, w;

    constexpr Vec4 operator+(const Vec4 &v) const { return Vec4{x + v.x, y + v.y, z + v.z, w + v.w}; }
    constexpr Vec4 operator*(const Vec4 &v) const { return Vec4{x * v.x, y * v.y, z * v.z, w * v.w}; }
    constexpr Vec4 operator*(const float f) const { return Vec4{x * f, y * f, z * f, w * f}; }
    constexpr Vec4 operator/(const float f) const { return *this * (1.0f / f); }
    constexpr float max() const { return std::max(std::max(x, y), z); }
};

struct Vec3
{
    float x, y, z;

    constexpr Vec3 operator-(const Vec3 &v) const { return Vec3{x - v.x, y - v.y, z - v.z}; }
    constexpr Vec3 operator+(const Vec3 &v) const { return Vec3{x + v.x, y + v.y, z + v.z}; }
    constexpr Vec3 operator*(const Vec3 &v) const { return Vec3{x * v.x, y * v.y, z * v.z}; }
    constexpr Vec3 operator*(const float f) const { return Vec3{x * f, y * f, z * f}; }
    constexpr Vec3 operator/(const float f) const { return *this * (1.0f / f); }
    constexpr Vec3 &operator+=(const Vec3 &v) { return *this = *this + v; }

    float length() const { return std::sqrt(x * x + y * y + z * z); }
    Vec3 normalized() const
    {
        const float l = length();
        return Vec3{x / l, y / l, z / l};
    }
    constexpr Vec3 cross(const Vec3 &v) const { return Vec3{y * v.z - z * v.y, z * v.x - x * v.z, x * v.y - y * v.x}; }
    constexpr float dot(const Vec3 &v) const { return x * v.x + y * v.y + z * v.z; }
    bool anyNan() const { return std::isnan(x) || std::isnan(y) || std::isnan(z); }
    constexpr Vec3 inv() const { return Vec3{1 / x, 1 / y, 1 / z}; }
};

template <typename T>
struct Vec2
{
    T x, y;

    constexpr Vec2 operator+(const Vec2 &v) const { return Vec2{x + v.x, y + v.y}; }
    constexpr Vec2 operator-(const Vec2 &v) const { return Vec2{x - v.x, y - v.y}; }
    constexpr Vec2 operator/(const Vec2 &v) const { return Vec2{x / v.x, y / v.y}; }
    constexpr Vec2 operator*(const Vec2 &v) const { return Vec2{x * v.x, y * v.y}; }
    constexpr Vec2 operator*(const T &f) const { return Vec2{x * f, y * f}; }
    constexpr Vec2 operator/(const T &f) const { return Vec2{x / f, y / f}; }

    template <typename U>
    constexpr operator Vec2<U>() const
    {
        return Vec2<U>{static_cast<U>(x), static_cast<U>(y)};
    }
};

using Vec2i = Vec2<int>;
using Vec2f = Vec2<float>;

template <typename T>
struct Size2
{
    T width, height;

    constexpr Size2 operator/(const T &v) const { return Size2{width / v, height / v}; }
    constexpr T area() const { return width * height; }
    constexpr Vec2<T> toVec() const { return Vec2<T>{width, height}; }
};

using Size2i = Size2<int>;
using Size2f = Size2<float>;

struct AABB
{
    Vec3 min, max;

    static constexpr AABB empty()
    {
        const float m = std::numeric_limits<float>::max();
        return AABB{Vec3{m, m, m}, Vec3{-m, -m, -m}};
    }
    constexpr AABB extend(const Vec3 &p) const
    {
        return AABB{Vec3{std::min(min.x, p.x), std::min(min.y, p.y), std::min(min.z, p.z)},
                    Vec3{std::max(max.x, p.x), std::max(max.y, p.y), std::max(max.z, p.z)}};
    }
};

struct Ray
{
    Vec3 p, v;
};

inline std::ostream &operator<<(std::ostream &os, const Vec3 &v) { return os << "(" << v.x << ", " << v.y << ", " << v.z << ")"; }
inline std::ostream &operator<<(std::ostream &os, const Vec4 &v)
{
    return os << "(" << v.x << ", " << v.y << ", " << v.z << ", " << v.w << ")";
}
template <typename T>
std::ostream &operator<<(std::ostream &os, const Size2<T> &s) { return os << "(" << s.width << ", " << s.height << ")"; }
template <typename T>
std::ostream &operator<<(std::ostream &os, const Vec2<T> &v) { return os << "(" << v.x << ", " << v.y << ")"; }

template <class... Ts>
struct Overloaded : Ts... {
    using Ts::operator()...;
};
template <class... Ts>
Overloaded(Ts...) -> Overloaded<Ts...>;

// Half the length of (A - B) x (A - C).
inline float triangleArea(const Vec3 &A, const Vec3 &B, const Vec3 &C) { return (A - B).cross(A - C).length() / 2; }

// Rec. 709 luminance of linear RGB.
constexpr float luminance(const Vec4 &c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

constexpr float powerHeuristic(const float pdf_0, const float pdf_1)
{
    return pdf_0 * pdf_0 / (pdf_0 * pdf_0 + pdf_1 * pdf_1);
}
