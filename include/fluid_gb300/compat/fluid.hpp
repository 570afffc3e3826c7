// fluid.hpp (compat) -- source-compatible stand-ins for libfluid's public types, for
// builds without GLM.  Same namespaces, struct names, fields and constructors as
// tom91136/libfluid include/fluid/fluid.hpp:13-232 and geometry.hpp:17-79; the vector
// type is a minimal glm::tvec3 with x/y/z members.  Code that already has the real
// libfluid headers (and GLM) includes those instead and gets the same adapter.
#ifndef LIBFLUID_FLUID_HPP
#define LIBFLUID_FLUID_HPP

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <ostream>
#include <vector>

namespace glm {
template <typename T>
struct tvec3 {
    T x{}, y{}, z{};
    tvec3() = default;
    explicit tvec3(T s) : x(s), y(s), z(s) {}
    tvec3(T x, T y, T z) : x(x), y(y), z(z) {}
    tvec3 operator+(const tvec3 &o) const { return {x + o.x, y + o.y, z + o.z}; }
    tvec3 operator-(const tvec3 &o) const { return {x - o.x, y - o.y, z - o.z}; }
    tvec3 operator*(T s) const { return {x * s, y * s, z * s}; }
    tvec3 operator/(T s) const { return {x / s, y / s, z / s}; }
    bool operator==(const tvec3 &o) const { return x == o.x && y == o.y && z == o.z; }
};
template <typename T>
struct tvec4 {
    T x{}, y{}, z{}, w{};
};
template <typename T>
inline T distance(const tvec3<T> &a, const tvec3<T> &b) {
    const tvec3<T> d = a - b;
    return std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
}
}  // namespace glm

namespace geometry {
using glm::tvec3;

template <typename N>
struct Triangle {
    tvec3<N> v0, v1, v2;
    Triangle() = default;
    explicit Triangle(const tvec3<N> &v0, const tvec3<N> &v1, const tvec3<N> &v2) : v0(v0), v1(v1), v2(v2) {}
};

template <typename N>
struct MeshTriangle {
    tvec3<N> v0, v1, v2;
    tvec3<N> n0, n1, n2;
    tvec3<uint32_t> c;
    MeshTriangle() = default;
    explicit MeshTriangle(const tvec3<N> &v0, const tvec3<N> &v1, const tvec3<N> &v2, const tvec3<N> &n0,
                          const tvec3<N> &n1, const tvec3<N> &n2)
        : v0(v0), v1(v1), v2(v2), n0(n0), n1(n1), n2(n2) {}
};
}  // namespace geometry

namespace fluid {
using glm::tvec3;
using glm::tvec4;

enum Type { Fluid = 0, Obstacle = 1 };

template <typename N>
struct Query {
    size_t id;
    tvec3<N> point;
};

template <typename N>
struct QueryResult {
    size_t id;
    tvec3<N> point;
    size_t neighbours;
    uint32_t averageColour;
    explicit QueryResult(size_t id, tvec3<N> point, size_t neighbours, uint32_t averageColour)
        : id(id), point(point), neighbours(neighbours), averageColour(averageColour) {}
};

template <typename T, typename N>
struct Particle {
    T id;
    Type type;
    N mass;
    tvec3<N> position;
    tvec3<N> velocity;
    uint32_t colour;
    Particle() : type(Type::Fluid) {}
    explicit Particle(T t, Type type, N mass, const uint32_t &colour, const tvec3<N> &position,
                      const tvec3<N> &velocity)
        : id(t), type(type), mass(mass), position(position), velocity(velocity), colour(colour) {}
};

template <typename N>
struct MeshCollider {
    const std::vector<geometry::Triangle<N>> triangles;
    explicit MeshCollider(const std::vector<geometry::Triangle<N>> &triangles) : triangles(triangles) {}
};

template <typename N>
struct Well {
    tvec3<N> centre;
    N force;
};

template <typename N>
struct Source {
    tvec3<N> centre;
    tvec3<N> velocity;
    size_t rate, tag;
    uint32_t colour;
};

template <typename N>
struct Drain {
    tvec3<N> centre;
    N width, depth;
};

template <typename N>
struct Config {
    const N dt;
    const N scale;
    const N resolution;
    const N isolevel;
    const size_t iteration;
    const tvec3<N> constantForce;
    const std::vector<fluid::Well<N>> wells;
    const std::vector<fluid::Source<N>> sources;
    const std::vector<fluid::Drain<N>> drains;
    const std::vector<fluid::Query<N>> queries;
    const tvec3<N> minBound, maxBound;
    explicit Config(N dt, N scale, N resolution, N isolevel, size_t iteration, const tvec3<N> &constantForce,
                    const std::vector<fluid::Well<N>> &wells, const std::vector<fluid::Source<N>> &sources,
                    const std::vector<fluid::Drain<N>> &drains, const std::vector<fluid::Query<N>> &queries,
                    const tvec3<N> &min, const tvec3<N> &max)
        : dt(dt), scale(scale), resolution(resolution), isolevel(isolevel), iteration(iteration),
          constantForce(constantForce), wells(wells), sources(sources), drains(drains), queries(queries),
          minBound(min), maxBound(max) {}
};

template <typename N>
struct Result {
    std::vector<geometry::MeshTriangle<N>> triangles{};
    std::vector<QueryResult<N>> queries{};
    Result() = default;
    Result(const std::vector<geometry::MeshTriangle<N>> &triangles, const std::vector<QueryResult<N>> &queries)
        : triangles(triangles), queries(queries) {}
};

template <typename T, typename N>
class SphSolver {
public:
    virtual ~SphSolver() = default;
    virtual Result<N> advance(const Config<N> &config, std::vector<Particle<T, N>> &xs,
                              const std::vector<MeshCollider<N>> &colliders) = 0;
};

}  // namespace fluid

#endif  // LIBFLUID_FLUID_HPP
