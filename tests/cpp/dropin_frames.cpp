// Times the drop-in as a libfluid application calls it: cuda::SphSolver::advance on a
// std::vector<fluid::Particle<size_t, float>> (samples/main.cpp:442), frame after
// frame.  bench.py writes the scene (the particles as records of the Particle layout,
// then the config) to a file; this program reads it, runs `warmup` untimed and
// `frames` timed frames, and prints one JSON line with the mean milliseconds a frame
// and a checksum of the final state.
//
//   dropin_frames <scene file> <warmup> <frames> <profile: 0 ref, 1 baseline>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fluid_gb300/compat/fluid.hpp"
#include "fluid_gb300/cudasph.hpp"

namespace {
// scene file: u64 n; then n records {u64 id; i32 type; f32 mass; f32 pos[3];
// f32 vel[3]; u32 colour; u32 pad} (48 bytes); then f32 dt, scale, resolution,
// isolevel; u32 iterations; f32 g[3], min[3], max[3], sphere[4] (radius 0: none)
struct Record {
    uint64_t id;
    int32_t type;
    float mass, pos[3], vel[3];
    uint32_t colour, pad;
};
static_assert(sizeof(Record) == 48, "record layout");
}  // namespace

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s scene warmup frames profile\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    uint64_t n = 0;
    if (std::fread(&n, 8, 1, f) != 1) return 4;
    std::vector<Record> recs(n);
    if (std::fread(recs.data(), sizeof(Record), n, f) != n) return 4;
    float head[4], g[3], mn[3], mx[3], sphere[4];
    uint32_t iterations = 0;
    if (std::fread(head, 4, 4, f) != 4 || std::fread(&iterations, 4, 1, f) != 1 || std::fread(g, 4, 3, f) != 3 ||
        std::fread(mn, 4, 3, f) != 3 || std::fread(mx, 4, 3, f) != 3 || std::fread(sphere, 4, 4, f) != 4)
        return 4;
    std::fclose(f);
    using fluid::tvec3;
    std::vector<fluid::Particle<size_t, float>> xs;
    xs.reserve(n);
    for (const Record &r : recs)
        xs.emplace_back((size_t)r.id, r.type ? fluid::Type::Obstacle : fluid::Type::Fluid, r.mass, r.colour,
                        tvec3<float>(r.pos[0], r.pos[1], r.pos[2]), tvec3<float>(r.vel[0], r.vel[1], r.vel[2]));
    const fluid::Config<float> config(head[0], head[1], head[2], head[3], iterations, tvec3<float>(g[0], g[1], g[2]),
                                      {}, {}, {}, {}, tvec3<float>(mn[0], mn[1], mn[2]),
                                      tvec3<float>(mx[0], mx[1], mx[2]));
    const int warmup = std::atoi(argv[2]), frames = std::atoi(argv[3]);
    cuda::SphSolver solver(0.1f, std::atoi(argv[4]) ? FGB_PROFILE_BASELINE : FGB_PROFILE_REF);
    solver.sphere(sphere[0], sphere[1], sphere[2], sphere[3]);
    const std::vector<fluid::MeshCollider<float>> colliders;
    fluid::SphSolver<size_t, float> &s = solver;
    for (int k = 0; k < warmup; ++k) s.advance(config, xs, colliders);
    const auto t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < frames; ++k) s.advance(config, xs, colliders);
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    double sp = 0;
    for (const auto &p : xs) sp += (double)p.position.x + 2.0 * p.position.y + 3.0 * p.position.z;
    std::printf("{\"n\": %llu, \"frames\": %d, \"ms_per_frame\": %.6f, \"pos_checksum\": %.9g}\n",
                (unsigned long long)n, frames, 1e3 * sec / frames, sp);
    return 0;
}
