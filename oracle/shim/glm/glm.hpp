// Minimal stand-in for the parts of glm's public API that the reference's
// geometry_util.cuh uses (vec<3, T>, +, -, scalar *, dot, cross, length,
// normalize, acos), so that file compiles from its own source for the
// oracle's pinning tests.  Written from glm's documented semantics (plain
// component-wise vector arithmetic); TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cmath>

namespace glm {

enum qualifier { defaultp = 0 };

template <int N, typename T, qualifier Q = defaultp>
struct vec;

template <typename T, qualifier Q>
struct vec<3, T, Q>
{
    T x, y, z;
    vec() : x(0), y(0), z(0) {}
    vec(T a, T b, T c) : x(a), y(b), z(c) {}
    T&       operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <typename T, qualifier Q>
inline vec<3, T, Q> operator-(const vec<3, T, Q>& a, const vec<3, T, Q>& b)
{
    return vec<3, T, Q>(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <typename T, qualifier Q>
inline vec<3, T, Q> operator+(const vec<3, T, Q>& a, const vec<3, T, Q>& b)
{
    return vec<3, T, Q>(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <typename T, qualifier Q>
inline vec<3, T, Q> operator*(T s, const vec<3, T, Q>& a)
{
    return vec<3, T, Q>(s * a.x, s * a.y, s * a.z);
}
template <typename T, qualifier Q>
inline vec<3, T, Q> operator/(const vec<3, T, Q>& a, T s)
{
    return vec<3, T, Q>(a.x / s, a.y / s, a.z / s);
}
template <typename T, qualifier Q>
inline T dot(const vec<3, T, Q>& a, const vec<3, T, Q>& b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T, qualifier Q>
inline vec<3, T, Q> cross(const vec<3, T, Q>& a, const vec<3, T, Q>& b)
{
    return vec<3, T, Q>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <typename T, qualifier Q>
inline T length(const vec<3, T, Q>& a)
{
    return std::sqrt(dot(a, a));
}
template <typename T, qualifier Q>
inline vec<3, T, Q> normalize(const vec<3, T, Q>& a)
{
    return a / length(a);
}
template <typename T>
inline T acos(T x)
{
    return std::acos(x);
}

}  // namespace glm
