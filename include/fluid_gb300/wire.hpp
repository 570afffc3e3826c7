// wire.hpp -- packed record streams for users of the C++ drop-in (cuda::SphSolver).
//
// Header-only writers with the meaning of strucures::writeParticles /
// writeTriangles / writeQueries (samples/structures.hpp:392-424) for the
// source-compatible fluid types, into any writable byte range (a memory-mapped
// file, a pinned buffer, a std::vector<char>).  The byte layout is the one the C ABI
// documents beside FGB_WIRE_HEADER_BYTES: header {int64 timestamp_ms, uint64
// entries, uint64 written}, then each record's fields in declaration order with no
// padding, little-endian; `written` is set last.  Each writer returns the bytes
// used, or throws std::length_error when `capacity` is too small.
#pragma once

#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "compat/fluid.hpp"
#include "../fluid_gb300.h"

namespace cuda {
namespace wire {

inline int64_t now_ms() {
    using namespace std::chrono;
    return duration_cast<milliseconds>(system_clock::now().time_since_epoch()).count();
}

namespace detail {
template <typename T>
inline unsigned char *put(unsigned char *p, const T &v) {
    std::memcpy(p, &v, sizeof v);
    return p + sizeof v;
}
template <typename N>
inline unsigned char *put3(unsigned char *p, const glm::tvec3<N> &v) {
    return put(put(put(p, v.x), v.y), v.z);
}
inline void header(void *dst, int64_t ts, uint64_t entries, uint64_t written) {
    unsigned char *p = static_cast<unsigned char *>(dst);
    if (written) std::atomic_thread_fence(std::memory_order_release);
    put(put(put(p, ts), entries), written);
}
template <typename R, typename F>
inline size_t stream(void *dst, size_t capacity, const std::vector<R> &xs, size_t record_bytes, int64_t ts, F &&pack) {
    const size_t need = FGB_WIRE_HEADER_BYTES + record_bytes * xs.size();
    if (capacity < need) throw std::length_error("wire: destination smaller than the stream");
    header(dst, ts, xs.size(), 0);
    unsigned char *p = static_cast<unsigned char *>(dst) + FGB_WIRE_HEADER_BYTES;
    for (const R &x : xs) p = pack(p, x);
    header(dst, ts, xs.size(), xs.size());
    return need;
}
}  // namespace detail

inline size_t particles_bytes(size_t n) { return FGB_WIRE_HEADER_BYTES + FGB_WIRE_PARTICLE_BYTES * n; }
inline size_t triangles_bytes(size_t n) { return FGB_WIRE_HEADER_BYTES + FGB_WIRE_TRIANGLE_BYTES * n; }
inline size_t queries_bytes(size_t n) { return FGB_WIRE_HEADER_BYTES + FGB_WIRE_QUERY_BYTES * n; }

// particle: u64 id, i32 type, f32 mass, u32 colour, f32 position[3], f32 velocity[3]
inline size_t writeParticles(void *dst, size_t capacity, const std::vector<fluid::Particle<size_t, float>> &xs,
                             int64_t ts = now_ms()) {
    return detail::stream(dst, capacity, xs, FGB_WIRE_PARTICLE_BYTES, ts,
                          [](unsigned char *p, const fluid::Particle<size_t, float> &x) {
                              p = detail::put(p, static_cast<uint64_t>(x.id));
                              p = detail::put(p, static_cast<int32_t>(x.type));
                              p = detail::put(p, x.mass);
                              p = detail::put(p, x.colour);
                              p = detail::put3(p, x.position);
                              return detail::put3(p, x.velocity);
                          });
}

// triangle: f32 v0, v1, v2, n0, n1, n2 (each [3]), u32 c[3]
inline size_t writeTriangles(void *dst, size_t capacity, const std::vector<geometry::MeshTriangle<float>> &xs,
                             int64_t ts = now_ms()) {
    return detail::stream(dst, capacity, xs, FGB_WIRE_TRIANGLE_BYTES, ts,
                          [](unsigned char *p, const geometry::MeshTriangle<float> &t) {
                              p = detail::put3(detail::put3(detail::put3(p, t.v0), t.v1), t.v2);
                              p = detail::put3(detail::put3(detail::put3(p, t.n0), t.n1), t.n2);
                              return detail::put3(p, t.c);
                          });
}

// query: u64 id, f32 point[3], u64 neighbours, u32 averageColour
inline size_t writeQueries(void *dst, size_t capacity, const std::vector<fluid::QueryResult<float>> &xs,
                           int64_t ts = now_ms()) {
    return detail::stream(dst, capacity, xs, FGB_WIRE_QUERY_BYTES, ts,
                          [](unsigned char *p, const fluid::QueryResult<float> &q) {
                              p = detail::put(p, static_cast<uint64_t>(q.id));
                              p = detail::put3(p, q.point);
                              p = detail::put(p, static_cast<uint64_t>(q.neighbours));
                              return detail::put(p, q.averageColour);
                          });
}

}  // namespace wire
}  // namespace cuda
