// glm/glm.hpp -- a project-written subset of the GLM vector API (TEST INFRASTRUCTURE:
// the timed reference arm only).  GLM itself is an external library the reference
// takes from vcpkg (README.md:30, version unpinned, not vendored) and is absent here.
// This subset holds what include/fluid/fluid.hpp, geometry.hpp and cpusph.hpp use:
// tvec3 / tvec4 with component-wise arithmetic, indexing and equality; distance,
// length, length2, dot, cross, normalize, min, max, pi, to_string, triangleNormal.
// The arithmetic is GLM's published definitions in single precision: dot(a, b) =
// (a.x*b.x + a.y*b.y) + a.z*b.z, length(v) = sqrt(dot(v, v)), distance(a, b) =
// length(b - a), normalize(v) = v * (1 / length(v)), min/max component-wise.
#ifndef FGB_GLM_SUBSET_HPP
#define FGB_GLM_SUBSET_HPP

#include <cmath>
#include <cstddef>
#include <string>

namespace glm {

template <typename T>
struct tvec3 {
    T x, y, z;
    tvec3() : x(0), y(0), z(0) {}
    explicit tvec3(T v) : x(v), y(v), z(v) {}
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <typename U>
    explicit tvec3(const tvec3<U> &o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    T &operator[](size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T &operator[](size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
    tvec3 &operator+=(const tvec3 &o) { x += o.x, y += o.y, z += o.z; return *this; }
    tvec3 &operator-=(const tvec3 &o) { x -= o.x, y -= o.y, z -= o.z; return *this; }
    tvec3 &operator*=(T s) { x *= s, y *= s, z *= s; return *this; }
    tvec3 &operator/=(T s) { x /= s, y /= s, z /= s; return *this; }
    tvec3 &operator+=(T s) { x += s, y += s, z += s; return *this; }
    tvec3 &operator-=(T s) { x -= s, y -= s, z -= s; return *this; }
    bool operator==(const tvec3 &o) const { return x == o.x && y == o.y && z == o.z; }
    bool operator!=(const tvec3 &o) const { return !(*this == o); }
};

template <typename T>
struct tvec4 {
    T x, y, z, w;
    tvec4() : x(0), y(0), z(0), w(0) {}
    explicit tvec4(T v) : x(v), y(v), z(v), w(v) {}
    tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    tvec4 &operator+=(const tvec4 &o) { x += o.x, y += o.y, z += o.z, w += o.w; return *this; }
};

template <typename T> tvec3<T> operator+(tvec3<T> a, const tvec3<T> &b) { return a += b; }
template <typename T> tvec3<T> operator-(tvec3<T> a, const tvec3<T> &b) { return a -= b; }
template <typename T> tvec3<T> operator-(const tvec3<T> &a) { return tvec3<T>(-a.x, -a.y, -a.z); }
template <typename T> tvec3<T> operator*(const tvec3<T> &a, const tvec3<T> &b) { return tvec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename T> tvec3<T> operator/(const tvec3<T> &a, const tvec3<T> &b) { return tvec3<T>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <typename T> tvec3<T> operator*(tvec3<T> a, T s) { return a *= s; }
template <typename T> tvec3<T> operator*(T s, const tvec3<T> &a) { return tvec3<T>(s * a.x, s * a.y, s * a.z); }
template <typename T> tvec3<T> operator/(tvec3<T> a, T s) { return a /= s; }
template <typename T> tvec3<T> operator+(tvec3<T> a, T s) { return a += s; }
template <typename T> tvec3<T> operator-(tvec3<T> a, T s) { return a -= s; }
template <typename T> tvec4<T> operator/(const tvec4<T> &a, T s) { return tvec4<T>(a.x / s, a.y / s, a.z / s, a.w / s); }

template <typename T> T pi() { return static_cast<T>(3.14159265358979323846264338327950288); }
template <typename T> T dot(const tvec3<T> &a, const tvec3<T> &b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <typename T> tvec3<T> cross(const tvec3<T> &a, const tvec3<T> &b) {
    return tvec3<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <typename T> T length2(const tvec3<T> &v) { return dot(v, v); }
template <typename T> T length(const tvec3<T> &v) { return std::sqrt(dot(v, v)); }
template <typename T> T distance(const tvec3<T> &a, const tvec3<T> &b) { return length(b - a); }
template <typename T> tvec3<T> normalize(const tvec3<T> &v) { return v * (static_cast<T>(1) / length(v)); }
template <typename T> tvec3<T> min(const tvec3<T> &a, const tvec3<T> &b) {
    return tvec3<T>(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z);
}
template <typename T> tvec3<T> max(const tvec3<T> &a, const tvec3<T> &b) {
    return tvec3<T>(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z);
}
template <typename T> tvec3<T> floor(const tvec3<T> &v) { return tvec3<T>(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
template <typename T> tvec3<T> triangleNormal(const tvec3<T> &a, const tvec3<T> &b, const tvec3<T> &c) {
    return normalize(cross(a - b, a - c));
}
template <typename T> std::string to_string(const tvec3<T> &v) {
    return "vec3(" + std::to_string(v.x) + ", " + std::to_string(v.y) + ", " + std::to_string(v.z) + ")";
}
template <typename T> std::string to_string(const tvec4<T> &v) {
    return "vec4(" + std::to_string(v.x) + ", " + std::to_string(v.y) + ", " + std::to_string(v.z) + ", " +
           std::to_string(v.w) + ")";
}

}  // namespace glm

#endif
