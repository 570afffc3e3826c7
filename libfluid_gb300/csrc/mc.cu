// mc.cu -- marching cubes on the device: field sampling, case classification fused
// into a decoupled-look-back prefix sum, and emission at scanned offsets.
//
// Reference: mc_lattice / mc_size / mc_eval (include/fluid/oclsph_kernel.h:421-735)
// with a host round trip for the triangle total (oclsph.hpp:450-465) and an
// atomic_inc append whose order is nondeterministic (oclsph_kernel.h:713).  Here
// the total stays on the device until the caller needs it, and triangles land in
// cube-major order with each cube's triangles in table order -- the order of the
// reference's CPU marchSingle loop (surface.hpp:185-266), whose edge lerp with its
// 1e-5 snapping (surface.hpp:47-53) is what the emit kernel evaluates.
//
// Layout of the work: the field kernel samples bricks of lattice nodes whose warps
// share grid cells; the classification runs over 16 consecutive cubes per scan
// thread; the emit kernel lets each warp gather its cubes that have triangles and
// write their triangles as whole 128-byte lines.
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "fgb_internal.h"
#include "mc_tables.h"
#include "scan.cuh"

namespace fgb {

__device__ uint16_t g_mc_edge_mask[256];
__device__ uint8_t g_mc_num_verts[256];
__device__ uint8_t g_mc_tri[256][16];

void mc_tables_upload() {
    fgb_mc_tables t;
    fgb_mc_tables_build(&t);
    cudaMemcpyToSymbol(g_mc_edge_mask, t.edge_mask, sizeof t.edge_mask);
    cudaMemcpyToSymbol(g_mc_num_verts, t.num_verts, sizeof t.num_verts);
    cudaMemcpyToSymbol(g_mc_tri, t.tri, sizeof t.tri);
}

namespace {

// Scene owning a global lattice sample, cube or field brick (scenes sorted by base).
enum class Base { kSample, kCube, kBrick };

template <Base B>
__device__ __forceinline__ uint32_t find_scene(const SceneDev *scenes, uint32_t lo, uint32_t hi, uint64_t q) {
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        const SceneDev &S = scenes[mid];
        const uint64_t base = B == Base::kCube ? S.cube_base : B == Base::kBrick ? S.brick_base : S.lat_base;
        if (base <= q) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t argb_channel(uint32_t c, int ch) { return (c >> (24 - 8 * ch)) & 0xffu; }

__device__ __forceinline__ uint32_t argb_pack(const float *ch) {
    uint32_t out = 0;
    for (int i = 0; i < 4; ++i) {
        float v = ch[i];
        if (!(v > 0.f)) v = 0.f;
        if (v > 255.f) v = 255.f;
        out |= ((uint32_t)v & 0xffu) << (24 - 8 * i);
    }
    return out;
}

// The particles of the 27 cells around (cx, cy, cz) in walk order as f(b, x_b), with
// the positions of a cell's candidates loaded four at a time ahead of the tests.
template <class F>
__device__ __forceinline__ void field_walk(const SceneDev &S, const uint2 *__restrict__ cells,
                                           const float4 *__restrict__ xs, int cx, int cy, int cz, F &&f) {
    const uint2 *tbl = cells + S.table_base;
    for_cell_indices(S, cx, cy, cz, [&](uint32_t k) {
        const uint2 c = __ldg(&tbl[k]);
        uint32_t b = c.x;
        for (; b + 4 <= c.y; b += 4) {
            const float4 p0 = __ldg(&xs[b]), p1 = __ldg(&xs[b + 1]), p2 = __ldg(&xs[b + 2]), p3 = __ldg(&xs[b + 3]);
            f(b, p0);
            f(b + 1, p1);
            f(b + 2, p2);
            f(b + 3, p3);
        }
        for (; b < c.y; ++b) f(b, __ldg(&xs[b]));
    });
}

// Field value, normal and colour sums of one lattice node over its 27 cells.  kUnit:
// the scene's scale is 1, so x_b / scale is x_b itself and the divisions are skipped
// (the same values).  The range test comes before the obstacle test (both must pass)
// so that only candidates in range load their type.
template <int PROFILE, bool kUnit>
__device__ __forceinline__ void field_sums(const SceneDev &S, const Phys &ph, const uint2 *__restrict__ cells,
                                           const float4 *__restrict__ xs, const int32_t *__restrict__ type,
                                           const uint32_t *__restrict__ col, const int *cc, const float *node,
                                           float *acc, uint32_t *cl, uint32_t &N) {
    const float aw[3] = {node[0] * S.scale, node[1] * S.scale, node[2] * S.scale};
    float v = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
    field_walk(S, cells, xs, cc[0], cc[1], cc[2], [&](uint32_t b, const float4 &xb) {
        if (PROFILE == FGB_PROFILE_REF) {
            const float lx = xb.x - aw[0], ly = xb.y - aw[1], lz = xb.z - aw[2];
            const float r2 = lx * lx + ly * ly + lz * lz;
            if (!(r2 < S.mc_r2_lt)) return;  // sqrtf(r2) >= h * scale
            if (S.obstacles && __ldg(&type[b]) == FGB_TYPE_OBSTACLE) return;
            const float len = sqrtf(r2);
            const float den = (ph.mc_infl == 0.5f) ? sqrtf(len) : powf(len, ph.mc_infl);
            const float sc = (-ph.mc_infl * ph.mc_size) / den;
            nx = __fmaf_rn(sc, lx, nx);
            ny = __fmaf_rn(sc, ly, ny);
            nz = __fmaf_rn(sc, lz, nz);
            v = v + ph.mc_size / den;
        } else {
            float ax, ay, az;
            if (kUnit) ax = xb.x, ay = xb.y, az = xb.z;
            else ax = xb.x / S.scale, ay = xb.y / S.scale, az = xb.z / S.scale;
            const float dx = node[0] - ax, dy = node[1] - ay, dz = node[2] - az;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 <= ph.hh)) return;
            if (S.obstacles && __ldg(&type[b]) == FGB_TYPE_OBSTACLE) return;
            const float t = ph.hh - r2;
            const float mt = xb.w * (t * t);
            v = __fmaf_rn(mt, t, v);
            nx = __fmaf_rn(mt, dx, nx);
            ny = __fmaf_rn(mt, dy, ny);
            nz = __fmaf_rn(mt, dz, nz);
        }
        const uint32_t c = __ldg(&col[b]);
        for (int ch = 0; ch < 4; ++ch) cl[ch] += argb_channel(c, ch);
        N++;
    });
    acc[0] = v;
    acc[1] = nx;
    acc[2] = ny;
    acc[3] = nz;
}

// Whether any cell within one cell of the warp's nodes' cells holds a particle.  The
// nodes of a warp lie in a few adjacent cells, so the lanes share the table lookups of
// that common neighbourhood (at most 128 cells; larger ones are not checked).  When
// every cell is empty, every node's walk finds no candidate and its sums stay zero.
__device__ __forceinline__ bool warp_cells_occupied(const SceneDev &S, const uint2 *__restrict__ cells,
                                                    unsigned act, const int *cc) {
    uint32_t lo[3], n[3];
    for (int a = 0; a < 3; ++a) {
        const uint32_t mn = __reduce_min_sync(act, (uint32_t)cc[a]), mx = __reduce_max_sync(act, (uint32_t)cc[a]);
        lo[a] = mn > 0 ? mn - 1 : 0;
        n[a] = (mx < S.ext[a] ? mx + 1 : S.ext[a]) - lo[a] + 1;
    }
    const uint32_t total = n[0] * n[1] * n[2];
    if (total > 128u) return true;
    const uint2 *tbl = cells + S.table_base;
    const uint32_t r = __popc(act & lanemask_lt()), cnt = __popc(act);
    bool any = false;
    for (uint32_t k = r; k < total; k += cnt) {
        const uint32_t x = lo[0] + k % n[0], y = lo[1] + (k / n[0]) % n[1], z = lo[2] + k / (n[0] * n[1]);
        const uint2 c = __ldg(&tbl[spread10(x) | (spread10(y) << 1) | (spread10(z) << 2)]);
        any |= c.x < c.y;
    }
    return __any_sync(act, any);
}

// One CTA per brick of kBrickX x kBrickY x kBrickZ lattice nodes of one scene; every
// node's value is its own walk's, whatever the thread that computes it.
template <int PROFILE>
__global__ void __launch_bounds__(256)
    k_field(const SceneDev *__restrict__ scenes, uint32_t scene_begin, uint32_t scene_end, Phys ph,
            const uint2 *__restrict__ cells, const float4 *__restrict__ xs, const int32_t *__restrict__ type,
            const uint32_t *__restrict__ col, uint64_t brick_begin, float4 *__restrict__ lattice,
            uint32_t *__restrict__ lattice_col) {
    const uint64_t brick = brick_begin + blockIdx.x;
    const uint32_t s = find_scene<Base::kBrick>(scenes, scene_begin, scene_end, brick);
    const SceneDev &S = scenes[s];
    // 32-bit index arithmetic: a scene's bricks and cubes number below 2^32
    const uint32_t local = (uint32_t)(brick - S.brick_base);
    const uint32_t nby = (S.lat[1] + kBrickY - 1) / kBrickY, nbz = (S.lat[2] + kBrickZ - 1) / kBrickZ;
    const uint32_t bz = local % nbz, by = (local / nbz) % nby, bx = local / (nbz * nby);
    const uint32_t w = threadIdx.x >> 5, l = threadIdx.x & 31u;
    const uint32_t ix = bx * kBrickX + (w & 1u) * 2u + (l & 1u);
    const uint32_t iy = by * kBrickY + ((w >> 1) & 1u) * 4u + ((l >> 1) & 3u);
    const uint32_t iz = bz * kBrickZ + (w >> 2) * 4u + (l >> 3);
    const bool valid = ix < S.lat[0] && iy < S.lat[1] && iz < S.lat[2];
    const float node[3] = {S.lat_origin[0] + (float)ix * S.lat_step, S.lat_origin[1] + (float)iy * S.lat_step,
                           S.lat_origin[2] + (float)iz * S.lat_step};
    int cc[3] = {0, 0, 0};
    if (valid) {
        if (PROFILE == FGB_PROFILE_REF) {
            const uint32_t id[3] = {ix, iy, iz};
            for (int a = 0; a < 3; ++a) {
                uint32_t c = (uint32_t)((float)id[a] / S.resolution);
                cc[a] = (int)(c > S.ext[a] ? S.ext[a] : c);
            }
        } else {
            for (int a = 0; a < 3; ++a) cc[a] = (int)quantise(node[a], S.min_ext[a], ph.h, S.ext[a]);
        }
    }
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    if (!valid) return;
    const uint64_t q = S.lat_base + ((uint64_t)ix * S.lat[1] + iy) * S.lat[2] + iz;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    // channel sums as integers: below 2^24, so equal to the float sums in any order
    uint32_t cl[4] = {0, 0, 0, 0};
    uint32_t N = 0;
    if (warp_cells_occupied(S, cells, act, cc)) {
        if (S.scale == 1.f) field_sums<PROFILE, true>(S, ph, cells, xs, type, col, cc, node, acc, cl, N);
        else field_sums<PROFILE, false>(S, ph, cells, xs, type, col, cc, node, acc, cl, N);
    }
    float v = acc[0], nx = acc[1], ny = acc[2], nz = acc[3];
    if (PROFILE != FGB_PROFILE_REF) v = v * ph.poly6f;
    const float nl = sqrtf(nx * nx + ny * ny + nz * nz);
    if (nl > 0.f) {
        nx = nx / nl;
        ny = ny / nl;
        nz = nz / nl;
    }
    lattice[q] = make_float4(v, nx, ny, nz);
    float avg[4] = {0.f, 0.f, 0.f, 0.f};
    if (N)
        for (int ch = 0; ch < 4; ++ch) avg[ch] = (float)cl[ch] / (float)N;
    lattice_col[q] = argb_pack(avg);
}

// Scan loader: classify cubes `cube_begin + i`, record their cases, return their
// triangle counts.
struct CubeCount {
    const SceneDev *scenes;
    uint32_t scene_begin, scene_end;
    const float4 *lattice;
    uint8_t *cases;
    uint64_t cube_begin;
    // Cubes first .. first + K - 1 (those below n): the scene and the cube's
    // coordinates are found once and then stepped, and a cube that follows another
    // along z takes its four corners on the plane between them from that cube's case,
    // loading four lattice values instead of eight.
    template <int K>
    __device__ __forceinline__ void run(uint64_t first, uint64_t n, uint32_t (&v)[K]) const {
        const SceneDev *S = nullptr;
        uint64_t row = 0, plane = 0;  // lattice index of (x, y, 0); samples per x-plane
        uint32_t sz = 0, mx = 0, my = 0, mz = 0, x = 0, y = 0, z = 0, prev = 0;
        bool have = false;
        float iso = 0.f;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            v[k] = 0u;
            const uint64_t i = first + k;
            if (i >= n) continue;
            if (!S || x >= mx) {  // first cube, or past the end of a scene's cubes
                const uint64_t q = cube_begin + i;
                S = &scenes[find_scene<Base::kCube>(scenes, scene_begin, scene_end, q)];
                const uint32_t local = (uint32_t)(q - S->cube_base);
                mx = S->lat[0] - 1;
                my = S->lat[1] - 1;
                mz = S->lat[2] - 1;
                x = local / (my * mz);
                y = (local / mz) % my;
                z = local % mz;
                sz = S->lat[2];
                plane = (uint64_t)S->lat[1] * sz;
                row = S->lat_base + (uint64_t)x * plane + (uint64_t)y * sz;
                iso = S->iso;
                have = false;
            }
            const uint64_t r00 = row + z, r10 = r00 + plane, r01 = r00 + sz, r11 = r10 + sz;
            auto below = [&](uint64_t idx, int bit) { return __ldg(&lattice[idx].x) < iso ? 1u << bit : 0u; };
            uint32_t ci = have ? prev >> 4 : below(r00, 0) | below(r10, 1) | below(r11, 2) | below(r01, 3);
            ci |= below(r00 + 1, 4) | below(r10 + 1, 5) | below(r11 + 1, 6) | below(r01 + 1, 7);
            prev = ci;
            cases[i] = (uint8_t)ci;
            v[k] = g_mc_edge_mask[ci] ? (uint32_t)(g_mc_num_verts[ci] / 3) : 0u;
            have = true;
            if (++z == mz) {
                z = 0;
                have = false;
                row += sz;
                if (++y == my) {
                    y = 0;
                    ++x;
                    row = S->lat_base + (uint64_t)x * plane;
                }
            }
        }
    }
};

// surface.hpp:47-53 compares |d| (a float widened to double) with the double 0.00001;
// `snap` is the smallest float not below that double, so |d| < snap is the same test
// without double arithmetic.
__device__ __forceinline__ int snap_select(float iso, float v1, float v2, float snap) {
    if (fabsf(iso - v1) < snap) return 1;
    if (fabsf(iso - v2) < snap) return 2;
    if (fabsf(v1 - v2) < snap) return 1;
    return 0;
}

// Corner c of a cube as (x, y, z) offsets and edge e as its two corners, in the
// reference's numbering (surface.hpp): constant expressions, so that unrolled loops
// index the corner registers directly.
__host__ __device__ constexpr uint32_t corner_x(int c) { return ((c + 1) >> 1) & 1; }
__host__ __device__ constexpr uint32_t corner_y(int c) { return (c >> 1) & 1; }
__host__ __device__ constexpr uint32_t corner_z(int c) { return c >> 2; }
__host__ __device__ constexpr int edge_a(int e) { return e < 8 ? e : e - 8; }
__host__ __device__ constexpr int edge_b(int e) { return e < 8 ? ((e & 4) | ((e + 1) & 3)) : e - 4; }

constexpr int kEmitWarps = 4, kEmitCubesPerLane = 4;
constexpr int kEmitCubes = kEmitWarps * 32 * kEmitCubesPerLane;  // cubes per CTA
constexpr int kEdgeWords = 12 * 7 + 1;  // per lane: 12 edge vertices (position, normal, colour), padded

// Triangles of the cubes [i0, i0 + kEmitCubes) at their scanned offsets.  Each warp
// takes 128 cubes, lists those that have triangles (in cube order), and handles them 32
// at a time: a lane computes one cube's edge vertices into shared memory, then the
// warp writes the group's triangles -- contiguous in the output, since the offsets are
// an exclusive scan in cube order -- word by word, 32 consecutive words per store.
__global__ void __launch_bounds__(kEmitWarps * 32)
    k_emit(const SceneDev *__restrict__ scenes, uint32_t scene_begin, uint32_t scene_end,
           const float4 *__restrict__ lattice, const uint32_t *__restrict__ lattice_col,
           const uint8_t *__restrict__ cases, const uint32_t *__restrict__ offsets, uint64_t cube_begin,
           uint64_t cubes, fgb_mesh_triangle *__restrict__ out, uint64_t cap, float snap, uint32_t *err) {
    __shared__ float s_edge[kEmitWarps][32][kEdgeWords];
    __shared__ uint8_t s_act[kEmitWarps][32 * kEmitCubesPerLane];
    __shared__ uint8_t s_owner[kEmitWarps][32 * 5], s_which[kEmitWarps][32 * 5];
    __shared__ uint8_t s_case[kEmitWarps][32];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t i0 = (uint64_t)blockIdx.x * kEmitCubes + (uint64_t)w * 32 * kEmitCubesPerLane;
    // this warp's cubes that have triangles, in cube order
    uint32_t n_act = 0;
#pragma unroll
    for (int k = 0; k < kEmitCubesPerLane; ++k) {
        const uint64_t i = i0 + 32u * k + lane;
        const bool on = i < cubes && g_mc_edge_mask[cases[i]] != 0;
        const unsigned m = __ballot_sync(0xffffffffu, on);
        if (on) s_act[w][n_act + __popc(m & lanemask_lt())] = (uint8_t)(32u * k + lane);
        n_act += __popc(m);
    }
    __syncwarp();
    float *ed = s_edge[w][lane];
    for (uint32_t g = 0; g < n_act; g += 32) {
        const bool mine = g + lane < n_act;
        const uint64_t i = i0 + (mine ? s_act[w][g + lane] : s_act[w][g]);
        const uint32_t ci = cases[i];
        const uint32_t ntri = mine ? g_mc_num_verts[ci] / 3 : 0u;
        // the group's triangles start at the offset of its first cube
        uint32_t incl = ntri;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t tri_total = __shfl_sync(0xffffffffu, incl, 31);
        const uint64_t t0 = offsets[i0 + s_act[w][g]];
        if (mine) {
            s_case[w][lane] = (uint8_t)ci;
            for (uint32_t t = 0; t < ntri; ++t) {
                s_owner[w][incl - ntri + t] = (uint8_t)lane;
                s_which[w][incl - ntri + t] = (uint8_t)t;
            }
            const uint64_t q = cube_begin + i;
            const uint32_t s = find_scene<Base::kCube>(scenes, scene_begin, scene_end, q);
            const SceneDev &S = scenes[s];
            const uint32_t local = (uint32_t)(q - S.cube_base);
            const uint32_t my = S.lat[1] - 1, mz = S.lat[2] - 1;
            const uint32_t x = local / (my * mz), y = (local / mz) % my, z = local % mz;
            const uint64_t sy = S.lat[1], sz = S.lat[2];
            const float iso = S.iso;
            float val[8], pw[8][3], nrm[8][3];
            uint32_t col[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const uint32_t ox = x + corner_x(c), oy = y + corner_y(c), oz = z + corner_z(c);
                const uint64_t idx = S.lat_base + ((uint64_t)ox * sy + oy) * sz + oz;
                const float4 L = __ldg(&lattice[idx]);
                val[c] = L.x;
                nrm[c][0] = L.y;
                nrm[c][1] = L.z;
                nrm[c][2] = L.w;
                col[c] = __ldg(&lattice_col[idx]);
                pw[c][0] = ((float)ox * S.lat_step + S.lat_origin[0]) * S.scale;
                pw[c][1] = ((float)oy * S.lat_step + S.lat_origin[1]) * S.scale;
                pw[c][2] = ((float)oz * S.lat_step + S.lat_origin[2]) * S.scale;
            }
            const uint16_t em = g_mc_edge_mask[ci];
#pragma unroll
            for (int e = 0; e < 12; ++e) {
                if (!(em & (1u << e))) continue;
                const int a = edge_a(e), b = edge_b(e);
                float *o = ed + 7 * e;
                const int sel = snap_select(iso, val[a], val[b], snap);
                if (sel) {
                    const bool first = sel == 1;
                    for (int d = 0; d < 3; ++d) {
                        o[d] = first ? pw[a][d] : pw[b][d];
                        o[3 + d] = first ? nrm[a][d] : nrm[b][d];
                    }
                    o[6] = __uint_as_float(first ? col[a] : col[b]);
                } else {
                    const float mu = (iso - val[a]) / (val[b] - val[a]);
                    for (int d = 0; d < 3; ++d) {
                        o[d] = pw[a][d] + (pw[b][d] - pw[a][d]) * mu;
                        o[3 + d] = nrm[a][d] + (nrm[b][d] - nrm[a][d]) * mu;
                    }
                    float ch[4];
                    for (int c = 0; c < 4; ++c) {
                        const float fa = (float)argb_channel(col[a], c), fb = (float)argb_channel(col[b], c);
                        ch[c] = fa + (fb - fa) * mu;
                    }
                    o[6] = __uint_as_float(argb_pack(ch));
                }
            }
        }
        __syncwarp();
        // the group's triangles, 21 words each, written in order
        if (t0 + tri_total > cap) {
            if (lane == 0) raise_error(err, ERR_MESH_CAPACITY);
        } else {
            uint32_t *dst = reinterpret_cast<uint32_t *>(out + t0);
            for (uint32_t wd = lane; wd < 21u * tri_total; wd += 32) {
                const uint32_t t = wd / 21u, f = wd - 21u * t;
                const uint32_t owner = s_owner[w][t], tt = s_which[w][t];
                const uint32_t vert = f < 18u ? (f < 9u ? f / 3u : (f - 9u) / 3u) : f - 18u;
                const uint32_t e = g_mc_tri[s_case[w][owner]][3u * tt + vert];
                const uint32_t comp = f < 9u ? f % 3u : f < 18u ? 3u + (f - 9u) % 3u : 6u;
                dst[wd] = __float_as_uint(s_edge[w][owner][7u * e + comp]);
            }
        }
        __syncwarp();
    }
}

}  // namespace

cudaError_t launch_surface_count(const SurfaceView &v, cudaStream_t st, uint64_t *launches) {
    const uint64_t bricks = v.brick_end - v.brick_begin;
    if (bricks) {
        const unsigned grid = (unsigned)bricks;
        if (v.ph.profile == FGB_PROFILE_REF)
            k_field<FGB_PROFILE_REF><<<grid, 256, 0, st>>>(v.scenes, v.scene_begin, v.scene_end, v.ph, v.cells, v.xs,
                                                          v.type, v.col, v.brick_begin, v.lattice,
                                                          v.lattice_col);
        else
            k_field<FGB_PROFILE_BASELINE><<<grid, 256, 0, st>>>(v.scenes, v.scene_begin, v.scene_end, v.ph, v.cells,
                                                               v.xs, v.type, v.col, v.brick_begin,
                                                               v.lattice, v.lattice_col);
        if (launches) *launches += 1;
    }
    CubeCount load{v.scenes, v.scene_begin, v.scene_end, v.lattice, v.cases, v.cube_begin};
    return scan_launch(load, v.offsets, v.total, v.cube_end - v.cube_begin, v.scan_scratch, v.scan_scratch_bytes,
                       st, v.err, launches);
}

// The smallest float whose widening to double is not below 0.00001.
static float snap_threshold() {
    float f = (float)0.00001;
    while ((double)f < 0.00001) f = std::nextafter(f, INFINITY);
    while ((double)std::nextafter(f, 0.f) >= 0.00001) f = std::nextafter(f, 0.f);
    return f;
}

cudaError_t launch_surface_emit(const SurfaceView &v, fgb_mesh_triangle *out, uint64_t cap, cudaStream_t st,
                                uint64_t *launches) {
    const uint64_t cubes = v.cube_end - v.cube_begin;
    if (!cubes || !cap) return cudaSuccess;
    k_emit<<<(unsigned)((cubes + kEmitCubes - 1) / kEmitCubes), kEmitWarps * 32, 0, st>>>(v.scenes, v.scene_begin, v.scene_end, v.lattice,
                                                           v.lattice_col, v.cases, v.offsets, v.cube_begin, cubes,
                                                           out, cap, snap_threshold(), v.err);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

}  // namespace fgb
