// Drives cuda::SphSolver exactly as the reference demo drives ocl::SphSolver
// (samples/main.cpp:398-442): a block of particles, a Config, advance per frame.
// Prints one JSON line the tests compare with the C ABI called from Python.
#include <cstdio>
#include <vector>

#include "fluid_gb300/compat/fluid.hpp"
#include "fluid_gb300/cudasph.hpp"

int main() {
    using fluid::tvec3;
    std::vector<fluid::Particle<size_t, float>> xs;
    size_t id = 0;
    for (int x = 0; x < 12; ++x)
        for (int y = 0; y < 12; ++y)
            for (int z = 0; z < 12; ++z)
                xs.emplace_back(id++, fluid::Type::Fluid, 1.f, 0xFF2D1010u,
                                tvec3<float>(0.025f + 0.05f * x, 0.025f + 0.05f * y, 0.025f + 0.05f * z),
                                tvec3<float>(0.f));
    const fluid::Config<float> config(0.0083f, 1.f, 2.f, 100.f, 4, tvec3<float>(0.f, -9.8f, 0.f), {}, {},
                                      {fluid::Drain<float>{tvec3<float>(5.f, 5.f, 5.f), 0.1f, 0.1f}},
                                      {fluid::Query<float>{7, tvec3<float>(0.3f, 0.05f, 0.3f)}},
                                      tvec3<float>(0.f), tvec3<float>(1.5f, 1.5f, 1.5f));
    cuda::SphSolver solver(0.1f);
    fluid::Result<float> result;
    for (int frame = 0; frame < 3; ++frame) result = solver.advance(config, xs, {});
    double sp = 0, sv = 0;
    unsigned long long sid = 0;
    for (const auto &p : xs) {
        sp += (double)p.position.x + 2.0 * p.position.y + 3.0 * p.position.z;
        sv += (double)p.velocity.x + 2.0 * p.velocity.y + 3.0 * p.velocity.z;
        sid = sid * 1000003ull + p.id;
    }
    const size_t qn = result.queries.empty() ? 0 : result.queries[0].neighbours;
    const unsigned qc = result.queries.empty() ? 0u : result.queries[0].averageColour;
    std::printf("{\"n\": %zu, \"pos\": %.9g, \"vel\": %.9g, \"id_hash\": %llu, \"triangles\": %zu, \"queries\": %zu, "
                "\"q_neighbours\": %zu, \"q_colour\": %u}\n",
                xs.size(), sp, sv, sid, result.triangles.size(), result.queries.size(), qn, qc);
    return 0;
}
