// edit.cu -- sources and drains of a resident scene, on the device.
//
// Reference: the CPU pass at the start of ocl::SphSolver::advance
// (include/fluid/oclsph.hpp:675-708): sources append particles, then every fluid
// particle closer than a drain's width to its centre is erased (erase-remove, so
// the survivors keep their order).  Here the drained particles are flagged by one
// kernel, the survivors' new places come from a prefix scan of the flags, and one
// scatter moves the state into the other buffer set, leaving a gap after the
// edited scene's survivors for the emitted particles (which the host generates,
// as they are few, and copies in).
#include <cuda_runtime.h>

#include "fgb_internal.h"

namespace fgb {
namespace {

// glm::distance(drain.centre, x.position) < drain.width (oclsph.hpp:699-702)
__global__ void k_drain_flags(uint64_t n, uint32_t mbits, uint32_t scene, const uint32_t *__restrict__ keys,
                              const float4 *__restrict__ x, const int32_t *__restrict__ type,
                              const fgb_drain *__restrict__ drains, uint32_t n_drains, uint32_t *__restrict__ keep) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t k = 1;
        if (scene_of(keys[i], mbits) == scene && type[i] != FGB_TYPE_OBSTACLE) {
            const float4 p = x[i];
            for (uint32_t d = 0; d < n_drains; ++d) {
                const fgb_drain dr = drains[d];
                const float dx = dr.centre[0] - p.x, dy = dr.centre[1] - p.y, dz = dr.centre[2] - p.z;
                if (sqrtf(dx * dx + dy * dy + dz * dz) < dr.width) {
                    k = 0;
                    break;
                }
            }
        }
        keep[i] = k;
    }
}

// Survivor i of scene s goes to rank[i], shifted by the emitted count when s lies
// after the edited scene.  The edited scene's survivors are renumbered (slot = place
// in the scene); every other scene keeps its slots, and its ids move with it.
__global__ void k_edit_scatter(uint64_t n, uint32_t mbits, uint32_t scene, uint64_t emitted,
                               const uint32_t *__restrict__ keys, const uint32_t *__restrict__ keep,
                               const uint32_t *__restrict__ rank, const SceneMove *__restrict__ moves,
                               const float4 *__restrict__ x0, const float4 *__restrict__ v0,
                               const int32_t *__restrict__ t0, const uint32_t *__restrict__ c0,
                               const uint32_t *__restrict__ s0, const uint64_t *__restrict__ ids0,
                               float4 *__restrict__ x1, float4 *__restrict__ v1, int32_t *__restrict__ t1,
                               uint32_t *__restrict__ c1, uint32_t *__restrict__ s1, uint64_t *__restrict__ ids1) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        const uint32_t s = scene_of(keys[i], mbits);
        const uint64_t j = rank[i] + (s > scene ? emitted : 0);
        const SceneMove m = moves[s];
        x1[j] = x0[i];
        v1[j] = v0[i];
        t1[j] = t0[i];
        c1[j] = c0[i];
        const uint64_t id = ids0[m.first_old + s0[i]];
        if (s == scene) {
            const uint32_t slot = (uint32_t)(j - m.first_new);
            s1[j] = slot;
            ids1[m.first_new + slot] = id;
        } else {
            s1[j] = s0[i];
            ids1[m.first_new + s0[i]] = id;
        }
    }
}

unsigned grid_of(uint64_t n) {
    uint64_t g = (n + 255) / 256;
    if (g > 152u * 8u) g = 152u * 8u;
    return g ? (unsigned)g : 1u;
}

}  // namespace

void launch_drain_flags(uint64_t n, uint32_t mbits, uint32_t scene, const uint32_t *keys, const float4 *x,
                        const int32_t *type, const fgb_drain *drains, uint32_t n_drains, uint32_t *keep,
                        cudaStream_t st) {
    if (n) k_drain_flags<<<grid_of(n), 256, 0, st>>>(n, mbits, scene, keys, x, type, drains, n_drains, keep);
}

void launch_edit_scatter(uint64_t n, uint32_t mbits, uint32_t scene, uint64_t emitted, const uint32_t *keys,
                         const uint32_t *keep, const uint32_t *rank, const SceneMove *moves, const float4 *x0,
                         const float4 *v0, const int32_t *t0, const uint32_t *c0, const uint32_t *s0,
                         const uint64_t *ids0, float4 *x1, float4 *v1, int32_t *t1, uint32_t *c1, uint32_t *s1,
                         uint64_t *ids1, cudaStream_t st) {
    if (n)
        k_edit_scatter<<<grid_of(n), 256, 0, st>>>(n, mbits, scene, emitted, keys, keep, rank, moves, x0, v0, t0, c0,
                                                    s0, ids0, x1, v1, t1, c1, s1, ids1);
}

}  // namespace fgb
