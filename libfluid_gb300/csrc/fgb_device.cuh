// fgb_device.cuh -- device-side building blocks shared by the PBF and MC kernels.
//
// All float arithmetic is written with an explicit operation order: the library is
// compiled with -fmad=false, and fused multiply-adds appear only as __fmaf_rn, so a
// kernel computes the same bits on every code path that evaluates the same sum.
// Where the CPU oracle uses fmaf the kernels do too, so the two round alike.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fgb {

// Error flag bits raised by kernels (read by fgb_batch_error_flags).
enum : uint32_t {
    ERR_SORT_LOOKBACK = 1u << 0,  // radix-sort look-back wait gave up
    ERR_SCAN_LOOKBACK = 1u << 1,  // prefix-scan look-back wait gave up
    ERR_CELL_RANGE = 1u << 2,     // a key outside its scene's cell table
    ERR_MESH_CAPACITY = 1u << 3,  // more triangles than the output buffer holds
    ERR_WELD_TABLE = 1u << 4,     // a vertex found no slot in the welding hash table
};

// Bound on every look-back spin: after this many polls the waiting CTA records an
// error flag and stops waiting, so a lost predecessor can never hang the GPU.
constexpr uint32_t kSpinLimit = 1u << 22;

// Look-back settings of one sort pass or scan launch, passed by value.  Normally
// skip_tile is ~0u and spin_limit kSpinLimit.  fgb_test_lookback_fault sets a tile
// that never publishes its status and a small spin limit, so that the tile after it
// runs out of polls, raises its error flag and returns: the tested form of a lost
// predecessor.
struct LookbackCtl {
    uint32_t skip_tile;
    uint32_t spin_limit;
};

constexpr float kKernelEpsilon = 0.00000001f;  // oclsph_kernel.h:24
constexpr float kPiF = 3.14159265358979323846f;

// 10 bits per axis, x in bit 0, y in bit 1, z in bit 2 (curves.h:56-72 layout).
__host__ __device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__host__ __device__ __forceinline__ uint32_t compact10(uint32_t v) {
    v &= 0x09249249u;
    v = (v ^ (v >> 2)) & 0x030c30c3u;
    v = (v ^ (v >> 4)) & 0x0300f00fu;
    v = (v ^ (v >> 8)) & 0xff0000ffu;
    v = (v ^ (v >> 16)) & 0x000003ffu;
    return v;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return spread10(x) | (spread10(y) << 1) | (spread10(z) << 2);
}

// Solver constants (fgb_params resolved to the values the kernels use).
struct Phys {
    float h, hh;
    float hh_le;      // the largest float r2 with sqrtf(r2) <= h: r2 <= hh_le is exactly sqrtf(r2) <= h
    float poly6f;     // 315 / (64 pi h^9)
    float spikyf;     // -45 / (pi h^6)
    float rho0, inv_rho0;
    float cfm;
    float corr_k;     // ref: k; baseline: k * h^2
    float corr_n;
    float corr_ref;   // ref: poly6(dq)
    float corr_wdq;   // baseline: (h^2 - dq^2)^3
    float inv_corr_ref, inv_corr_wdq;
    float xsph_c, vort_eps, damping;
    float mc_size, mc_infl;
    int profile;      // FGB_PROFILE_*
};

// One scene of a batch, as the kernels see it.
struct SceneDev {
    float min_ext[3];     // grid origin, solver units
    uint32_t ext[3];      // cells are clamped to [0, ext]
    uint32_t table_base;  // first entry of this scene's cell table
    uint32_t first, count;
    float dt, inv_dt, scale;
    float g[3];
    float min_b[3], max_b[3];
    int sphere_enabled;
    float sphere[4];
    uint32_t n_wells, well_first;
    uint32_t tri_first, tri_count;
    uint32_t obstacles;   // obstacle particles in the scene (0: neighbours need no type check)
    // marching cubes
    uint32_t lat[3];
    float lat_origin[3];
    float lat_step;
    float resolution;
    float iso;
    float mc_r2_lt;      // ref profile: sqrtf(r2) < h * scale exactly when r2 < mc_r2_lt
    uint64_t lat_base;   // first lattice sample of this scene
    uint64_t cube_base;  // first cube of this scene
    uint64_t brick_base; // first field brick (kBrick* samples) of this scene
};

// The field kernel's bricks: one CTA samples a 4 x 8 x 8 block of lattice nodes, each
// warp a 2 x 4 x 4 block of it, so that a warp's lanes share their grid cells.
constexpr uint32_t kBrickX = 4, kBrickY = 8, kBrickZ = 8;
__host__ __device__ inline uint64_t field_bricks(const uint32_t *lat) {
    if (!lat[0] || !lat[1] || !lat[2]) return 0;
    return (uint64_t)((lat[0] + kBrickX - 1) / kBrickX) * ((lat[1] + kBrickY - 1) / kBrickY) *
           ((lat[2] + kBrickZ - 1) / kBrickZ);
}

struct WellDev {
    float centre[3];
    float force;
};

struct TriDev {
    float a[3], b[3], c[3];
};

__device__ __forceinline__ void raise_error(uint32_t *flags, uint32_t bit) {
    if (flags) atomicOr(flags, bit);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Cell of a coordinate (solver units) on one axis: (v - min) / h truncated,
// clamped into [0, ext]; a negative or NaN quotient maps to 0 (oclsph.hpp:327-332
// casts it to size_t, which is undefined there).
__device__ __forceinline__ uint32_t quantise(float v, float mn, float h, uint32_t ext) {
    float q = __fdiv_rn(__fsub_rn(v, mn), h);
    if (!(q > 0.f)) return 0u;
    if (q >= (float)ext) return ext;
    return (uint32_t)q;
}

__device__ __forceinline__ uint32_t scene_of(uint32_t key, uint32_t mbits) {
    return mbits >= 32 ? 0u : (key >> mbits);
}
__device__ __forceinline__ uint32_t morton_of(uint32_t key, uint32_t mbits) {
    return mbits >= 32 ? key : (key & ((1u << mbits) - 1u));
}

// The next value of one axis's interleaved bits (mask m) of a Morton code: the bits
// of the other axes are set so that the carry runs through them, then cleared.
__device__ __forceinline__ uint32_t morton_inc(uint32_t s, uint32_t m) { return ((s | ~m) + 1u) & m; }

// The cell-table indices (within scene S's table) of the 27 cells around cell
// (cx, cy, cz), each coordinate in [0, ext], in the reference's order (z, then y, then
// x ascending: oclsph_kernel.h:155-183), as f(index); cells outside [0, ext] hold no
// particle and are left out.  The indices advance by Morton increments rather than
// interleaving every coordinate afresh.
template <class F>
__device__ __forceinline__ void for_cell_indices(const SceneDev &S, int cx, int cy, int cz, F &&f) {
    constexpr uint32_t kMX = 0x09249249u, kMY = kMX << 1, kMZ = kMX << 2;
    const int ex = (int)S.ext[0], ey = (int)S.ext[1], ez = (int)S.ext[2];
    const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx < ex ? cx + 1 : ex;
    const int y0 = cy > 0 ? cy - 1 : 0, y1 = cy < ey ? cy + 1 : ey;
    const int z0 = cz > 0 ? cz - 1 : 0, z1 = cz < ez ? cz + 1 : ez;
    const uint32_t sx0 = spread10((uint32_t)x0), sy0 = spread10((uint32_t)y0) << 1;
    uint32_t sz = spread10((uint32_t)z0) << 2;
    for (int z = z0; z <= z1; ++z, sz = morton_inc(sz, kMZ)) {
        uint32_t sy = sy0;
        for (int y = y0; y <= y1; ++y, sy = morton_inc(sy, kMY)) {
            const uint32_t yz = sy | sz;
            uint32_t sx = sx0;
            for (int x = x0; x <= x1; ++x, sx = morton_inc(sx, kMX)) f(sx | yz);
        }
    }
}

// Visit the particles of the 27 cells around cell (cx, cy, cz) of scene S in the
// reference's order, each cell in sorted order.
template <class F>
__device__ __forceinline__ void for_neighbour_cells(const SceneDev &S, const uint2 *__restrict__ cells, int cx,
                                                    int cy, int cz, F &&f) {
    const uint2 *tbl = cells + S.table_base;
    for_cell_indices(S, cx, cy, cz, [&](uint32_t k) {
        const uint2 c = __ldg(&tbl[k]);
        for (uint32_t b = c.x; b < c.y; ++b) f(b);
    });
}

}  // namespace fgb
