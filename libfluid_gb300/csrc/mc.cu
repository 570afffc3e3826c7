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

__constant__ uint8_t c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                       {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__constant__ uint8_t c_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                      {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

// Scene owning a global lattice sample / cube (scenes sorted by base).
__device__ __forceinline__ uint32_t find_scene(const SceneDev *scenes, uint32_t lo, uint32_t hi, uint64_t q,
                                               bool cubes) {
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        uint64_t base = cubes ? scenes[mid].cube_base : scenes[mid].lat_base;
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

template <int PROFILE>
__global__ void __launch_bounds__(256)
    k_field(const SceneDev *__restrict__ scenes, uint32_t scene_begin, uint32_t scene_end, Phys ph,
            const uint2 *__restrict__ cells, const float4 *__restrict__ xs, const int32_t *__restrict__ type,
            const uint32_t *__restrict__ col, uint64_t lat_begin, uint64_t lat_end, float4 *__restrict__ lattice,
            uint32_t *__restrict__ lattice_col) {
    const uint64_t q = lat_begin + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= lat_end) return;
    const uint32_t s = find_scene(scenes, scene_begin, scene_end, q, false);
    const SceneDev &S = scenes[s];
    const uint64_t local = q - S.lat_base;
    const uint64_t sy = S.lat[1], sz = S.lat[2];
    const uint32_t ix = (uint32_t)(local / (sy * sz)), iy = (uint32_t)((local / sz) % sy),
                   iz = (uint32_t)(local % sz);
    const float node[3] = {S.lat_origin[0] + (float)ix * S.lat_step, S.lat_origin[1] + (float)iy * S.lat_step,
                           S.lat_origin[2] + (float)iz * S.lat_step};
    int cc[3];
    if (PROFILE == FGB_PROFILE_REF) {
        const uint32_t id[3] = {ix, iy, iz};
        for (int a = 0; a < 3; ++a) {
            uint32_t c = (uint32_t)((float)id[a] / S.resolution);
            cc[a] = (int)(c > S.ext[a] ? S.ext[a] : c);
        }
    } else {
        for (int a = 0; a < 3; ++a) cc[a] = (int)quantise(node[a], S.min_ext[a], ph.h, S.ext[a]);
    }
    const float thr = ph.h * S.scale;
    const float aw[3] = {node[0] * S.scale, node[1] * S.scale, node[2] * S.scale};
    float v = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
    // channel sums as integers: below 2^24, so equal to the float sums in any order
    uint32_t cl[4] = {0, 0, 0, 0};
    uint32_t N = 0;
    for_neighbour_cells(S, cells, cc[0], cc[1], cc[2], [&](uint32_t b) {
        if (S.obstacles && __ldg(&type[b]) == FGB_TYPE_OBSTACLE) return;
        const float4 xb = __ldg(&xs[b]);
        if (PROFILE == FGB_PROFILE_REF) {
            const float lx = xb.x - aw[0], ly = xb.y - aw[1], lz = xb.z - aw[2];
            const float len = sqrtf(lx * lx + ly * ly + lz * lz);
            if (!(len < thr)) return;
            const float den = (ph.mc_infl == 0.5f) ? sqrtf(len) : powf(len, ph.mc_infl);
            const float sc = (-ph.mc_infl * ph.mc_size) / den;
            nx = __fmaf_rn(sc, lx, nx);
            ny = __fmaf_rn(sc, ly, ny);
            nz = __fmaf_rn(sc, lz, nz);
            v = v + ph.mc_size / den;
        } else {
            const float dx = node[0] - xb.x / S.scale, dy = node[1] - xb.y / S.scale, dz = node[2] - xb.z / S.scale;
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 <= ph.hh)) return;
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

// Scan loader: classify cube `cube_begin + i`, record its case, return its triangles.
struct CubeCount {
    const SceneDev *scenes;
    uint32_t scene_begin, scene_end;
    const float4 *lattice;
    uint8_t *cases;
    uint64_t cube_begin;
    __device__ __forceinline__ uint32_t operator()(uint64_t i) const {
        const uint64_t q = cube_begin + i;
        const uint32_t s = find_scene(scenes, scene_begin, scene_end, q, true);
        const SceneDev &S = scenes[s];
        const uint64_t local = q - S.cube_base;
        const uint64_t my = S.lat[1] - 1, mz = S.lat[2] - 1;
        const uint64_t x = local / (my * mz), y = (local / mz) % my, z = local % mz;
        const uint64_t sy = S.lat[1], sz = S.lat[2];
        uint32_t ci = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const uint64_t idx = S.lat_base + ((x + c_corner[c][0]) * sy + (y + c_corner[c][1])) * sz +
                                 (z + c_corner[c][2]);
            if (__ldg(&lattice[idx].x) < S.iso) ci |= 1u << c;
        }
        cases[i] = (uint8_t)ci;
        return g_mc_edge_mask[ci] ? (uint32_t)(g_mc_num_verts[ci] / 3) : 0u;
    }
};

__device__ __forceinline__ int snap_select(float iso, float v1, float v2) {
    if ((double)fabsf(iso - v1) < 0.00001) return 1;
    if ((double)fabsf(iso - v2) < 0.00001) return 2;
    if ((double)fabsf(v1 - v2) < 0.00001) return 1;
    return 0;
}

__global__ void __launch_bounds__(256)
    k_emit(const SceneDev *__restrict__ scenes, uint32_t scene_begin, uint32_t scene_end,
           const float4 *__restrict__ lattice, const uint32_t *__restrict__ lattice_col,
           const uint8_t *__restrict__ cases, const uint32_t *__restrict__ offsets, uint64_t cube_begin,
           uint64_t cubes, fgb_mesh_triangle *__restrict__ out, uint64_t cap, uint32_t *err) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cubes) return;
    const uint32_t ci = cases[i];
    if (!g_mc_edge_mask[ci]) return;
    const uint32_t nv = g_mc_num_verts[ci];
    const uint64_t o0 = offsets[i];
    if (o0 + nv / 3 > cap) {
        raise_error(err, ERR_MESH_CAPACITY);
        return;
    }
    const uint64_t q = cube_begin + i;
    const uint32_t s = find_scene(scenes, scene_begin, scene_end, q, true);
    const SceneDev &S = scenes[s];
    const uint64_t local = q - S.cube_base;
    const uint64_t my = S.lat[1] - 1, mz = S.lat[2] - 1;
    const uint64_t x = local / (my * mz), y = (local / mz) % my, z = local % mz;
    const uint64_t sy = S.lat[1], sz = S.lat[2];
    const float iso = S.iso;
    float val[8], pw[8][3], nrm[8][3];
    uint32_t col[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint64_t ox = x + c_corner[c][0], oy = y + c_corner[c][1], oz = z + c_corner[c][2];
        const uint64_t idx = S.lat_base + (ox * sy + oy) * sz + oz;
        const float4 L = lattice[idx];
        val[c] = L.x;
        nrm[c][0] = L.y;
        nrm[c][1] = L.z;
        nrm[c][2] = L.w;
        col[c] = lattice_col[idx];
        pw[c][0] = ((float)ox * S.lat_step + S.lat_origin[0]) * S.scale;
        pw[c][1] = ((float)oy * S.lat_step + S.lat_origin[1]) * S.scale;
        pw[c][2] = ((float)oz * S.lat_step + S.lat_origin[2]) * S.scale;
    }
    const uint16_t em = g_mc_edge_mask[ci];
    float ev[12][3], en[12][3];
    uint32_t ec[12];
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        if (!(em & (1u << e))) continue;
        const int a = c_edge[e][0], b = c_edge[e][1];
        const int sel = snap_select(iso, val[a], val[b]);
        if (sel) {
            const int k = sel == 1 ? a : b;
            for (int d = 0; d < 3; ++d) {
                ev[e][d] = pw[k][d];
                en[e][d] = nrm[k][d];
            }
            ec[e] = col[k];
        } else {
            const float mu = (iso - val[a]) / (val[b] - val[a]);
            for (int d = 0; d < 3; ++d) {
                ev[e][d] = pw[a][d] + (pw[b][d] - pw[a][d]) * mu;
                en[e][d] = nrm[a][d] + (nrm[b][d] - nrm[a][d]) * mu;
            }
            float ch[4];
            for (int c = 0; c < 4; ++c) {
                const float fa = (float)argb_channel(col[a], c), fb = (float)argb_channel(col[b], c);
                ch[c] = fa + (fb - fa) * mu;
            }
            ec[e] = argb_pack(ch);
        }
    }
    for (uint32_t t = 0; t < nv; t += 3) {
        fgb_mesh_triangle *m = &out[o0 + t / 3];
        for (int j = 0; j < 3; ++j) {
            const int e = g_mc_tri[ci][t + j];
            m->v[3 * j] = ev[e][0];
            m->v[3 * j + 1] = ev[e][1];
            m->v[3 * j + 2] = ev[e][2];
            m->n[3 * j] = en[e][0];
            m->n[3 * j + 1] = en[e][1];
            m->n[3 * j + 2] = en[e][2];
            m->c[j] = ec[e];
        }
    }
}

}  // namespace

cudaError_t launch_surface_count(const SurfaceView &v, cudaStream_t st, uint64_t *launches) {
    const uint64_t samples = v.lat_end - v.lat_begin;
    if (samples) {
        const unsigned grid = (unsigned)((samples + 255) / 256);
        if (v.ph.profile == FGB_PROFILE_REF)
            k_field<FGB_PROFILE_REF><<<grid, 256, 0, st>>>(v.scenes, v.scene_begin, v.scene_end, v.ph, v.cells, v.xs,
                                                          v.type, v.col, v.lat_begin, v.lat_end, v.lattice,
                                                          v.lattice_col);
        else
            k_field<FGB_PROFILE_BASELINE><<<grid, 256, 0, st>>>(v.scenes, v.scene_begin, v.scene_end, v.ph, v.cells,
                                                               v.xs, v.type, v.col, v.lat_begin, v.lat_end,
                                                               v.lattice, v.lattice_col);
        if (launches) *launches += 1;
    }
    CubeCount load{v.scenes, v.scene_begin, v.scene_end, v.lattice, v.cases, v.cube_begin};
    return scan_launch(load, v.offsets, v.total, v.cube_end - v.cube_begin, v.scan_scratch, v.scan_scratch_bytes,
                       st, v.err, launches);
}

cudaError_t launch_surface_emit(const SurfaceView &v, fgb_mesh_triangle *out, uint64_t cap, cudaStream_t st,
                                uint64_t *launches) {
    const uint64_t cubes = v.cube_end - v.cube_begin;
    if (!cubes || !cap) return cudaSuccess;
    k_emit<<<(unsigned)((cubes + 255) / 256), 256, 0, st>>>(v.scenes, v.scene_begin, v.scene_end, v.lattice,
                                                           v.lattice_col, v.cases, v.offsets, v.cube_begin, cubes,
                                                           out, cap, v.err);
    if (launches) *launches += 1;
    return cudaGetLastError();
}

}  // namespace fgb
