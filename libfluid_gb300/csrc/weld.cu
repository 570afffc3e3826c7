// weld.cu -- vertex welding of a triangle soup (an index buffer for rendering).
//
// Reference: geometry::indexVBO2 (include/fluid/geometry.hpp:152-166, unused by the
// solver): the vertices v0, v1, v2 of each triangle in order; a vertex whose
// position is byte-identical to an earlier one (PackedVertex compares with memcmp,
// geometry.hpp:81-88) takes that one's index, otherwise it is appended.  So the
// output is the distinct positions in order of first appearance, and every input
// vertex's index is the rank of its position's first appearance.
//
// On the device, order-free and deterministic:
//   k_weld_insert  each vertex i inserts its 12-byte position into an open-
//                  addressing table (a slot holds the index of the vertex that
//                  claimed it; keys are compared through the input positions) and
//                  lowers the slot's `first` to i with atomicMin
//   k_weld_first   first[i] = the minimum index of i's position; flag[i] = first == i
//   scan           rank of each flagged vertex (scan.cu)
//   k_weld_emit    index[i] = rank[first[i]], vertices[rank[i]] = position i if flagged
// The reference stores indices as unsigned short, which wraps after 65 535 distinct
// vertices; these are 32-bit.
#include <cstring>
#include <cuda_runtime.h>

#include "fgb_internal.h"

namespace fgb {
namespace {

constexpr uint32_t kEmpty = 0xffffffffu;

// Position of vertex i: triangle i / 3, corner i % 3, in the 21-word triangle record.
__device__ __forceinline__ uint3 vertex_bits(const float *tris, uint64_t i) {
    const float *p = tris + 21 * (i / 3) + 3 * (i % 3);
    return make_uint3(__float_as_uint(p[0]), __float_as_uint(p[1]), __float_as_uint(p[2]));
}

__device__ __forceinline__ uint32_t hash3(uint3 k) {
    uint32_t h = k.x * 0x9E3779B1u;
    h ^= (k.y + 0x7F4A7C15u + (h << 6) + (h >> 2)) * 0x85EBCA77u;
    h ^= (k.z + 0x165667B1u + (h << 6) + (h >> 2)) * 0xC2B2AE3Du;
    return h ^ (h >> 15);
}

__global__ void k_weld_insert(const float *__restrict__ tris, uint64_t nv, uint32_t mask, uint32_t *owner,
                              uint32_t *first, uint32_t *slot_of, uint32_t *err) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint3 key = vertex_bits(tris, i);
        uint32_t h = hash3(key) & mask;
        bool placed = false;
        // the table has at least twice as many slots as vertices, so a free or
        // matching slot is found within mask + 1 probes
        for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
            uint32_t o = atomicCAS(&owner[h], kEmpty, (uint32_t)i);
            if (o != kEmpty) {
                const uint3 other = vertex_bits(tris, o);
                if (other.x != key.x || other.y != key.y || other.z != key.z) continue;
            }
            atomicMin(&first[h], (uint32_t)i);
            slot_of[i] = h;
            placed = true;
            break;
        }
        if (!placed) {  // unreachable at load <= 1/2; keeps later passes in bounds
            slot_of[i] = 0;
            raise_error(err, ERR_WELD_TABLE);
        }
    }
}

__global__ void k_weld_first(uint64_t nv, const uint32_t *__restrict__ first, const uint32_t *__restrict__ slot_of,
                             uint32_t *__restrict__ first_of, uint32_t *__restrict__ flag) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t f = first[slot_of[i]];
        if (f > (uint32_t)i) f = (uint32_t)i;  // only after a table error: keep indices in range
        first_of[i] = f;
        flag[i] = f == (uint32_t)i ? 1u : 0u;
    }
}

__global__ void k_weld_emit(const float *__restrict__ tris, uint64_t nv, const uint32_t *__restrict__ first_of,
                            const uint32_t *__restrict__ flag, const uint32_t *__restrict__ rank,
                            uint32_t *__restrict__ index, float *__restrict__ vertices) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (uint64_t)gridDim.x * blockDim.x) {
        index[i] = rank[first_of[i]];
        if (flag[i]) {
            const float *p = tris + 21 * (i / 3) + 3 * (i % 3);
            float *o = vertices + 3 * (uint64_t)rank[i];
            o[0] = p[0];
            o[1] = p[1];
            o[2] = p[2];
        }
    }
}

template <class T>
struct Scratch {
    T *p = nullptr;
    cudaError_t alloc(uint64_t n) { return cudaMalloc((void **)&p, (n ? n : 1) * sizeof(T)); }
    ~Scratch() {
        if (p) cudaFree(p);
    }
};

unsigned grid_of(uint64_t n) {
    uint64_t g = (n + 255) / 256;
    if (g > 152u * 8u) g = 152u * 8u;
    return g ? (unsigned)g : 1u;
}

}  // namespace

// Weld the triangles at device address d_tris (21-word records).  Indices (3 per
// triangle) and the distinct vertices (3 floats each, at most 3 n) go to device
// memory; the vertex count to *n_vertices.
int weld_device(const fgb_mesh_triangle *d_tris, uint64_t n_tris, uint32_t *d_index, float *d_vertices,
                uint64_t *n_vertices, cudaStream_t st) {
    const uint64_t nv = 3 * n_tris;
    *n_vertices = 0;
    if (!nv) return FGB_OK;
    if (nv > 0x7fffffffull) return fail(FGB_ERR_CAPACITY, "weld: more than 2^31 vertices");
    uint64_t slots = 1;
    while (slots < 2 * nv) slots <<= 1;
    const float *tris = reinterpret_cast<const float *>(d_tris);
    Scratch<uint32_t> owner, first, slot_of, first_of, flag, rank, total, err;
    Scratch<char> scratch;
    const uint64_t sb = scan_u32_scratch_bytes(nv);
    cudaError_t e = owner.alloc(slots);
    if (e == cudaSuccess) e = first.alloc(slots);
    if (e == cudaSuccess) e = slot_of.alloc(nv);
    if (e == cudaSuccess) e = first_of.alloc(nv);
    if (e == cudaSuccess) e = flag.alloc(nv);
    if (e == cudaSuccess) e = rank.alloc(nv);
    if (e == cudaSuccess) e = total.alloc(1);
    if (e == cudaSuccess) e = err.alloc(1);
    if (e == cudaSuccess) e = scratch.alloc(sb);
    if (e != cudaSuccess) return fail(FGB_ERR_OOM, "weld: scratch allocation failed");
    e = cudaMemsetAsync(owner.p, 0xff, slots * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(first.p, 0xff, slots * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(err.p, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return fail_cuda(e, "weld: clear");
    k_weld_insert<<<grid_of(nv), 256, 0, st>>>(tris, nv, (uint32_t)(slots - 1), owner.p, first.p, slot_of.p, err.p);
    k_weld_first<<<grid_of(nv), 256, 0, st>>>(nv, first.p, slot_of.p, first_of.p, flag.p);
    e = scan_u32(flag.p, rank.p, total.p, nv, scratch.p, sb, st, err.p, nullptr);
    if (e == cudaSuccess) {
        k_weld_emit<<<grid_of(nv), 256, 0, st>>>(tris, nv, first_of.p, flag.p, rank.p, d_index, d_vertices);
        e = cudaGetLastError();
    }
    uint32_t t = 0, flags = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&t, total.p, sizeof t, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, err.p, sizeof flags, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda(e, "weld");
    if (flags) return fail(FGB_ERR_TIMEOUT, "weld: a device-side bound was hit (error flag set)");
    *n_vertices = t;
    return FGB_OK;
}

}  // namespace fgb

using fgb::fail;

extern "C" {

int fgb_weld_mesh(const fgb_mesh *mesh, uint32_t *indices, float *vertices, uint64_t *n_vertices) {
    if (!mesh || !n_vertices) return fail(FGB_ERR_INVALID, "weld_mesh: null argument");
    *n_vertices = 0;
    const uint64_t n = mesh->n, nv = 3 * n;
    if (!n) return FGB_OK;
    if (!mesh->triangles || !indices || !vertices) return fail(FGB_ERR_INVALID, "weld_mesh: null array");
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "weld_mesh: stream");
    fgb::Scratch<fgb_mesh_triangle> tris;
    fgb::Scratch<uint32_t> idx;
    fgb::Scratch<float> verts;
    int rc = FGB_OK;
    if (tris.alloc(n) != cudaSuccess || idx.alloc(nv) != cudaSuccess || verts.alloc(3 * nv) != cudaSuccess)
        rc = fail(FGB_ERR_OOM, "weld_mesh: allocation failed");
    if (!rc) {
        e = cudaMemcpyAsync(tris.p, mesh->triangles, n * sizeof(fgb_mesh_triangle), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) rc = fgb::fail_cuda(e, "weld_mesh: upload");
    }
    uint64_t count = 0;
    if (!rc) rc = fgb::weld_device(tris.p, n, idx.p, verts.p, &count, st);
    if (!rc) {
        e = cudaMemcpyAsync(indices, idx.p, nv * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && count)
            e = cudaMemcpyAsync(vertices, verts.p, 3 * count * sizeof(float), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = fgb::fail_cuda(e, "weld_mesh: download");
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (!rc) *n_vertices = count;
    return rc;
}

int fgb_batch_weld_surface(fgb_batch *b, uint32_t scene, uint32_t *indices, float *vertices, uint64_t *n_vertices) {
    if (!n_vertices) return fail(FGB_ERR_INVALID, "weld_surface: null count");
    *n_vertices = 0;
    fgb::ResidentScene r;
    int rc = fgb::batch_resident(b, scene, &r);
    if (rc) return rc;
    if (!r.tris) return fail(FGB_ERR_INVALID, "weld_surface: call fgb_batch_surface_all first");
    const uint64_t nv = 3 * r.tri_count;
    if (!nv) return FGB_OK;
    if (!indices || !vertices) return fail(FGB_ERR_INVALID, "weld_surface: null array");
    fgb::Scratch<uint32_t> idx;
    fgb::Scratch<float> verts;
    if (idx.alloc(nv) != cudaSuccess || verts.alloc(3 * nv) != cudaSuccess)
        return fail(FGB_ERR_OOM, "weld_surface: allocation failed");
    uint64_t count = 0;
    rc = fgb::weld_device(r.tris, r.tri_count, idx.p, verts.p, &count, r.stream);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(indices, idx.p, nv * sizeof(uint32_t), cudaMemcpyDeviceToHost, r.stream);
    if (e == cudaSuccess && count)
        e = cudaMemcpyAsync(vertices, verts.p, 3 * count * sizeof(float), cudaMemcpyDeviceToHost, r.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r.stream);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "weld_surface: download");
    *n_vertices = count;
    return FGB_OK;
}

}  // extern "C"
