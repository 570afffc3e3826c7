// query.cu -- cell queries against the grid of a scene's last step.
//
// The reference answers fluid::Config::queries on the host during advance
// (include/fluid/oclsph.hpp:770-791): for each query point it takes the grid cell
// of the point in the step's grid (the one built from the predicted positions),
// counts the fluid particles in that cell and averages their colours, as copied
// before the step's colour diffusion, in float (clutil::unpackARGB /
// clutil::packARGB, clutils.hpp:205-234), and returns a result only for points
// whose cell holds fluid.  Here one thread answers one query from the batch's cell
// table, which holds exactly that grid until the next step or surface.
#include <cuda_runtime.h>

#include "fgb_internal.h"

namespace fgb {
namespace {

__global__ void k_query(const SceneDev *__restrict__ scenes, uint32_t scene, float h, const uint2 *__restrict__ cells,
                        const int32_t *__restrict__ type_sorted, const uint32_t *__restrict__ order,
                        const uint32_t *__restrict__ colour_prev, const fgb_query *__restrict__ q, uint32_t nq,
                        uint32_t *__restrict__ count, uint32_t *__restrict__ argb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const SceneDev &S = scenes[scene];
    // cell of (point / scale - minExtent) / h, truncated (oclsph.hpp:772-775, 327-332);
    // a point outside the grid has no cell (the reference's cast of a negative float
    // to size_t is undefined)
    uint32_t c[3];
    bool inside = true;
    for (int a = 0; a < 3; ++a) {
        const float u = __fdiv_rn(__fsub_rn(__fdiv_rn(q[i].point[a], S.scale), S.min_ext[a]), h);
        if (!(u >= 0.f) || u >= (float)S.ext[a] + 1.f) {
            inside = false;
            c[a] = 0;
        } else {
            c[a] = (uint32_t)u;
        }
    }
    const uint32_t key = morton3(c[0], c[1], c[2]);
    // the reference's table holds morton(extent) entries and its last one has no end
    // (oclsph.hpp:744, 780: zIdx + 1 < gridTableN)
    const uint32_t table_n = morton3(S.ext[0], S.ext[1], S.ext[2]);
    uint32_t sum[4] = {0, 0, 0, 0}, n = 0;
    if (inside && key + 1 < table_n) {
        const uint2 r = cells[S.table_base + key];
        for (uint32_t b = r.x; b < r.y; ++b) {
            if (type_sorted[b] != FGB_TYPE_FLUID) continue;
            const uint32_t col = colour_prev[order[b]];
            for (int ch = 0; ch < 4; ++ch) sum[ch] += (col >> (24 - 8 * ch)) & 0xffu;
            ++n;
        }
    }
    uint32_t packed = 0;
    if (n) {
        // channel sums are integers below 2^24, exact in float in any order; the mean is
        // one IEEE division, then truncated to 8 bits
        for (int ch = 0; ch < 4; ++ch)
            packed |= ((uint32_t)__fdiv_rn((float)sum[ch], (float)n) & 0xffu) << (24 - 8 * ch);
    }
    count[i] = n;
    argb[i] = packed;
}

}  // namespace

void launch_queries(const SceneDev *scenes, uint32_t scene, float h, const uint2 *cells, const int32_t *type_sorted,
                    const uint32_t *order, const uint32_t *colour_prev, const fgb_query *q, uint32_t nq,
                    uint32_t *count, uint32_t *argb, cudaStream_t st) {
    if (!nq) return;
    k_query<<<(nq + 127) / 128, 128, 0, st>>>(scenes, scene, h, cells, type_sorted, order, colour_prev, q, nq, count,
                                             argb);
}

}  // namespace fgb
