// wire.cu -- packed record streams of particles and triangles.
//
// The reference demo streams results to memory-mapped files with
// mmf::writer::writePacked (include/fluid/mmf.hpp), field by field in the order of
// the definitions in samples/structures.hpp (particleDef, meshTriangleDef,
// headerDef), with no padding.  Here the same bytes are produced for host arrays
// (fgb_wire_particles / fgb_wire_triangles) and, for a resident scene, packed on the
// device by one kernel and moved to the destination in a single copy
// (fgb_batch_wire_particles); a scene's triangles are already in the 84-byte record
// layout on the device and are copied as they are (fgb_batch_wire_surface).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <cuda_runtime.h>

#include "fgb_internal.h"

namespace fgb {
namespace {

static_assert(sizeof(fgb_mesh_triangle) == FGB_WIRE_TRIANGLE_BYTES, "triangle record layout");

struct WireHeader {
    int64_t timestamp;
    uint64_t entries, written;
};
static_assert(sizeof(WireHeader) == FGB_WIRE_HEADER_BYTES, "header layout");

// The header says `written` = 0 until the records are in place.
void put_header(void *dst, int64_t ts, uint64_t entries, uint64_t written) {
    const WireHeader h{ts, entries, written};
    if (written) std::atomic_thread_fence(std::memory_order_release);
    memcpy(dst, &h, sizeof h);
}

int check_room(void *dst, uint64_t capacity, uint64_t need, uint64_t *bytes, const char *what) {
    if (!bytes) return fail(FGB_ERR_INVALID, what);
    *bytes = need;
    if (dst && capacity < need) return fail(FGB_ERR_INVALID, "wire: destination smaller than the stream");
    return FGB_OK;
}

// One 44-byte particle record per thread, as 11 words at word 6 + 11 i of the
// staging buffer (the header occupies words 0-5).
__global__ void k_pack_particles(uint64_t n, const float4 *__restrict__ x, const float4 *__restrict__ v,
                                 const int32_t *__restrict__ type, const uint32_t *__restrict__ col,
                                 const uint32_t *__restrict__ slot, const uint64_t *__restrict__ ids,
                                 uint32_t *__restrict__ out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float4 X = x[i], V = v[i];
        const uint64_t id = ids[slot[i]];
        uint32_t *r = out + 6 + 11 * i;
        r[0] = (uint32_t)id;
        r[1] = (uint32_t)(id >> 32);
        r[2] = (uint32_t)type[i];
        r[3] = __float_as_uint(X.w);
        r[4] = col[i];
        r[5] = __float_as_uint(X.x);
        r[6] = __float_as_uint(X.y);
        r[7] = __float_as_uint(X.z);
        r[8] = __float_as_uint(V.x);
        r[9] = __float_as_uint(V.y);
        r[10] = __float_as_uint(V.z);
    }
}

}  // namespace
}  // namespace fgb

using fgb::fail;

extern "C" {

int fgb_wire_particles(const fgb_particles *xs, int64_t ts, void *dst, uint64_t capacity, uint64_t *bytes) {
    if (!xs) return fail(FGB_ERR_INVALID, "wire_particles: null particles");
    const uint64_t n = xs->n;
    int rc = fgb::check_room(dst, capacity, FGB_WIRE_HEADER_BYTES + FGB_WIRE_PARTICLE_BYTES * n, bytes,
                             "wire_particles: null size");
    if (rc || !dst) return rc;
    if (n && (!xs->position || !xs->velocity || !xs->mass || !xs->type))
        return fail(FGB_ERR_INVALID, "wire_particles: null particle array");
    fgb::put_header(dst, ts, n, 0);
    unsigned char *p = static_cast<unsigned char *>(dst) + FGB_WIRE_HEADER_BYTES;
    for (uint64_t i = 0; i < n; ++i, p += FGB_WIRE_PARTICLE_BYTES) {
        const uint64_t id = xs->id ? xs->id[i] : i;
        const uint32_t colour = xs->colour ? xs->colour[i] : 0xffffffffu;
        memcpy(p, &id, 8);
        memcpy(p + 8, &xs->type[i], 4);
        memcpy(p + 12, &xs->mass[i], 4);
        memcpy(p + 16, &colour, 4);
        memcpy(p + 20, &xs->position[3 * i], 12);
        memcpy(p + 32, &xs->velocity[3 * i], 12);
    }
    fgb::put_header(dst, ts, n, n);
    return FGB_OK;
}

int fgb_wire_triangles(const fgb_mesh *mesh, int64_t ts, void *dst, uint64_t capacity, uint64_t *bytes) {
    if (!mesh) return fail(FGB_ERR_INVALID, "wire_triangles: null mesh");
    const uint64_t n = mesh->n;
    int rc = fgb::check_room(dst, capacity, FGB_WIRE_HEADER_BYTES + FGB_WIRE_TRIANGLE_BYTES * n, bytes,
                             "wire_triangles: null size");
    if (rc || !dst) return rc;
    if (n && !mesh->triangles) return fail(FGB_ERR_INVALID, "wire_triangles: null triangles");
    fgb::put_header(dst, ts, n, 0);
    if (n) memcpy(static_cast<char *>(dst) + FGB_WIRE_HEADER_BYTES, mesh->triangles, n * FGB_WIRE_TRIANGLE_BYTES);
    fgb::put_header(dst, ts, n, n);
    return FGB_OK;
}

int fgb_batch_wire_particles(fgb_batch *b, uint32_t scene, int64_t ts, void *dst, uint64_t capacity,
                             uint64_t *bytes) {
    fgb::ResidentScene r;
    int rc = fgb::batch_resident(b, scene, &r);
    if (rc) return rc;
    const uint64_t need = FGB_WIRE_HEADER_BYTES + FGB_WIRE_PARTICLE_BYTES * r.n;
    rc = fgb::check_room(dst, capacity, need, bytes, "wire_particles: null size");
    if (rc || !dst) return rc;
    fgb::put_header(dst, ts, r.n, 0);
    if (r.n) {
        uint32_t *stage = static_cast<uint32_t *>(fgb::batch_wire_scratch(b, need));
        if (!stage) return fail(FGB_ERR_OOM, "wire_particles: staging allocation failed");
        const unsigned grid = (unsigned)std::min<uint64_t>((r.n + 255) / 256, 152u * 8u);
        fgb::k_pack_particles<<<grid, 256, 0, r.stream>>>(r.n, r.x + r.first, r.v + r.first, r.type + r.first,
                                                          r.col + r.first, r.slot + r.first, r.ids + r.first, stage);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<char *>(dst) + FGB_WIRE_HEADER_BYTES,
                                reinterpret_cast<char *>(stage) + FGB_WIRE_HEADER_BYTES, need - FGB_WIRE_HEADER_BYTES,
                                cudaMemcpyDeviceToHost, r.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(r.stream);
        if (e != cudaSuccess) return fgb::fail_cuda(e, "wire_particles");
    }
    fgb::put_header(dst, ts, r.n, r.n);
    return FGB_OK;
}

int fgb_batch_wire_surface(fgb_batch *b, uint32_t scene, int64_t ts, void *dst, uint64_t capacity,
                           uint64_t *bytes) {
    fgb::ResidentScene r;
    int rc = fgb::batch_resident(b, scene, &r);
    if (rc) return rc;
    if (!r.tris) return fail(FGB_ERR_INVALID, "wire_surface: call fgb_batch_surface_all first");
    rc = fgb::check_room(dst, capacity, FGB_WIRE_HEADER_BYTES + FGB_WIRE_TRIANGLE_BYTES * r.tri_count, bytes,
                         "wire_surface: null size");
    if (rc || !dst) return rc;
    fgb::put_header(dst, ts, r.tri_count, 0);
    if (r.tri_count) {
        cudaError_t e = cudaMemcpyAsync(static_cast<char *>(dst) + FGB_WIRE_HEADER_BYTES, r.tris,
                                        r.tri_count * FGB_WIRE_TRIANGLE_BYTES, cudaMemcpyDeviceToHost, r.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(r.stream);
        if (e != cudaSuccess) return fgb::fail_cuda(e, "wire_surface");
    }
    fgb::put_header(dst, ts, r.tri_count, r.tri_count);
    return FGB_OK;
}

}  // extern "C"
