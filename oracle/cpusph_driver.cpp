// cpusph_driver.cpp -- the benchmark's timed reference arm (TEST INFRASTRUCTURE).
//
// Runs the reference's own OpenMP PBF solver, cpu::SphSolver
// (include/fluid/cpusph.hpp:75-240), from the copy oracle/patch_cpusph.py makes
// (return type and return statement patched, nothing else), with GLM replaced by
// the project-written subset in oracle/glm_subset and the reference's vendored
// nanoflann.  The solver keeps the reference's own constants (rho0 6378, CFM 600,
// velocity damping 0.49), searches neighbours within 2h with a k-d tree, and has no
// wells, colliders, colour diffusion or surface.  The particles live in a
// std::vector<fluid::Particle<size_t, float>> across calls, so a timed step is one
// call of advance() exactly as a libfluid application makes it.
#include <chrono>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

#include "glm/glm.hpp"
#define CURVE_UINT3_TYPE glm::tvec3<size_t>
#define CURVE_UINT3_CTOR(x, y, z) (glm::tvec3<size_t>((x), (y), (z)))
#include "fluid.hpp"
#include "cpusph.hpp"

namespace {
struct RefCpu {
    explicit RefCpu(float h) : solver(h) {}
    cpu::SphSolver<size_t, float> solver;
    std::vector<fluid::Particle<size_t, float>> xs;
};
}  // namespace

extern "C" {

void *refcpu_create(float h) { return new RefCpu(h); }

void refcpu_destroy(void *s) { delete static_cast<RefCpu *>(s); }

int refcpu_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

int refcpu_load(void *s, size_t n, const uint64_t *id, const int32_t *type, const float *mass, const float *pos,
                const float *vel, const uint32_t *colour) {
    RefCpu *r = static_cast<RefCpu *>(s);
    r->xs.resize(n);
    for (size_t i = 0; i < n; ++i)
        r->xs[i] = fluid::Particle<size_t, float>(
            (size_t)id[i], type[i] ? fluid::Obstacle : fluid::Fluid, mass[i], colour[i],
            glm::tvec3<float>(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
            glm::tvec3<float>(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]));
    return 0;
}

// cfg: dt, scale, iterations, constant force [3], min bound [3], max bound [3].
// Runs `steps` calls of advance() and returns their wall time in seconds.
double refcpu_advance(void *s, const float *cfg, int steps) {
    RefCpu *r = static_cast<RefCpu *>(s);
    const fluid::Config<float> config(cfg[0], cfg[1], 0.f, 0.f, (size_t)cfg[2],
                                      glm::tvec3<float>(cfg[3], cfg[4], cfg[5]), {}, {}, {}, {},
                                      glm::tvec3<float>(cfg[6], cfg[7], cfg[8]),
                                      glm::tvec3<float>(cfg[9], cfg[10], cfg[11]));
    const std::vector<fluid::MeshCollider<float>> colliders;
    fluid::SphSolver<size_t, float> &base = r->solver;
    const auto t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < steps; ++k) base.advance(config, r->xs, colliders);
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int refcpu_store(void *s, float *pos, float *vel) {
    RefCpu *r = static_cast<RefCpu *>(s);
    for (size_t i = 0; i < r->xs.size(); ++i) {
        for (int a = 0; a < 3; ++a) {
            pos[3 * i + a] = r->xs[i].position[a];
            vel[3 * i + a] = r->xs[i].velocity[a];
        }
    }
    return 0;
}
}
