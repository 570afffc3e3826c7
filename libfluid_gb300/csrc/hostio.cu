// hostio.cu -- particles moved between the caller's host arrays and a resident
// scene by kernels that address the host arrays directly.
//
// On a GPU that reads pageable memory through the host's page tables (Grace's
// coherent link: cudaDevAttrPageableMemoryAccessUsesHostPageTables), a kernel may
// load from and store to any array the caller allocated.  The packing the
// reference does on the host before its buffer writes (include/fluid/oclsph.hpp:
// 822-831, particles into the ClSphAtoms arrays) and the write-back after its
// read-back (oclsph.hpp:866-892) then run on the GPU: the array-of-structures positions and
// velocities are read as contiguous runs, regrouped through shared memory into the
// float4 layout of the device state, and the reverse on the way out, so that every
// warp access to host memory is a contiguous run of 4-byte words.
#include <cuda_runtime.h>

#include <algorithm>

#include "fgb_internal.h"

namespace fgb {
namespace {

constexpr unsigned kTile = 256;  // particles per CTA tile (= threads per CTA)

unsigned grid_of(uint64_t n) {
    uint64_t g = (n + kTile - 1) / kTile;
    if (g > 152u * 8u) g = 152u * 8u;
    return g ? (unsigned)g : 1u;
}

// Whether the caller's position and velocity arrays are 16-byte aligned: a full
// tile's positions and velocities are then 3 KB each at 16-byte boundaries.
__device__ __forceinline__ bool motion_vec(const HostParticlesIn &in) {
    return ((reinterpret_cast<uintptr_t>(in.position) | reinterpret_cast<uintptr_t>(in.velocity)) & 15u) == 0;
}

// The positions and velocities of particles base .. base + m - 1 into shared memory,
// as 16-byte loads for a full, aligned tile (fewer requests over the host link).
__device__ __forceinline__ void load_motion_tile(const HostParticlesIn &in, uint64_t base, uint32_t m, bool vec,
                                                 float *sp, float *sv) {
    const unsigned t = threadIdx.x;
    const float *pp = in.position + 3 * base, *pv = in.velocity + 3 * base;
    if (vec && m == kTile) {
        const float4 *p4 = reinterpret_cast<const float4 *>(pp), *v4 = reinterpret_cast<const float4 *>(pv);
        for (uint32_t j = t; j < 3 * kTile / 4; j += kTile) {
            reinterpret_cast<float4 *>(sp)[j] = p4[j];
            reinterpret_cast<float4 *>(sv)[j] = v4[j];
        }
    } else {
        for (uint32_t j = t; j < 3 * m; j += kTile) {
            sp[j] = pp[j];
            sv[j] = pv[j];
        }
    }
}

__global__ void __launch_bounds__(kTile) k_pack_from_host(HostParticlesIn in, uint64_t n, float4 *__restrict__ x,
                                                         float4 *__restrict__ v, int32_t *__restrict__ type,
                                                         uint32_t *__restrict__ col, uint32_t *__restrict__ slot,
                                                         uint64_t *__restrict__ ids, uint32_t *__restrict__ obstacles) {
    __shared__ __align__(16) float sp[3 * kTile], sv[3 * kTile];
    const unsigned t = threadIdx.x;
    uint32_t obst = 0;
    const bool vec = motion_vec(in);
    for (uint64_t base = (uint64_t)blockIdx.x * kTile; base < n; base += (uint64_t)gridDim.x * kTile) {
        const uint32_t m = (uint32_t)(n - base < kTile ? n - base : kTile);
        const uint64_t i = base + t;
        // this particle's scalar fields are in flight with the tile's vectors
        int32_t ty = 0;
        float ma = 0.f;
        uint32_t co = 0xffffffffu;
        uint64_t id = i;
        if (t < m) {
            ty = in.type[i];
            ma = in.mass[i];
            if (in.colour) co = in.colour[i];
            if (in.id) id = in.id[i];
        }
        load_motion_tile(in, base, m, vec, sp, sv);
        __syncthreads();
        if (t < m) {
            x[i] = make_float4(sp[3 * t], sp[3 * t + 1], sp[3 * t + 2], ma);
            v[i] = make_float4(sv[3 * t], sv[3 * t + 1], sv[3 * t + 2], 0.f);
            type[i] = ty;
            col[i] = co;
            slot[i] = (uint32_t)i;
            ids[i] = id;
            obst += ty == FGB_TYPE_OBSTACLE;
        }
        __syncthreads();
    }
    // one atomic per warp
    for (int o = 16; o; o >>= 1) obst += __shfl_xor_sync(0xffffffffu, obst, o);
    if ((t & 31) == 0 && obst) atomicAdd(obstacles, obst);
}

__global__ void __launch_bounds__(kTile) k_unpack_to_host(HostParticlesOut out, uint64_t n,
                                                         const float4 *__restrict__ x, const float4 *__restrict__ v,
                                                         const int32_t *__restrict__ type,
                                                         const uint32_t *__restrict__ col,
                                                         const uint32_t *__restrict__ slot,
                                                         const uint64_t *__restrict__ ids) {
    __shared__ float sp[3 * kTile], sv[3 * kTile];
    const unsigned t = threadIdx.x;
    for (uint64_t base = (uint64_t)blockIdx.x * kTile; base < n; base += (uint64_t)gridDim.x * kTile) {
        const uint32_t m = (uint32_t)(n - base < kTile ? n - base : kTile);
        if (t < m) {
            const uint64_t i = base + t;
            const float4 X = x[i], V = v[i];
            sp[3 * t] = X.x;
            sp[3 * t + 1] = X.y;
            sp[3 * t + 2] = X.z;
            sv[3 * t] = V.x;
            sv[3 * t + 1] = V.y;
            sv[3 * t + 2] = V.z;
            if (out.mass) out.mass[i] = X.w;
            if (out.type) out.type[i] = type[i];
            if (out.colour) out.colour[i] = col[i];
            if (out.id) {
                const uint32_t sl = slot[i];
                out.id[i] = sl < n ? ids[sl] : sl;
            }
        }
        __syncthreads();
        float *pp = out.position ? out.position + 3 * base : nullptr;
        float *pv = out.velocity ? out.velocity + 3 * base : nullptr;
        for (uint32_t j = t; j < 3 * m; j += kTile) {
            if (pp) pp[j] = sp[j];
            if (pv) pv[j] = sv[j];
        }
        __syncthreads();
    }
}

// An upload split by when the step needs each field: positions, velocities, masses
// and types feed the prediction and the sort (k_pack_motion, which also counts the
// obstacles into the scene table), colours, ids and upload slots only the reorder
// after the sort (k_pack_static, on a second stream while the prediction and the sort
// run).
__global__ void __launch_bounds__(kTile) k_pack_motion(HostParticlesIn in, uint64_t n, float4 *__restrict__ x,
                                                      float4 *__restrict__ v, int32_t *__restrict__ type,
                                                      uint32_t *__restrict__ obstacles) {
    __shared__ __align__(16) float sp[3 * kTile], sv[3 * kTile];
    const unsigned t = threadIdx.x;
    uint32_t obst = 0;
    const bool vec = motion_vec(in);
    for (uint64_t base = (uint64_t)blockIdx.x * kTile; base < n; base += (uint64_t)gridDim.x * kTile) {
        const uint32_t m = (uint32_t)(n - base < kTile ? n - base : kTile);
        // this particle's type and mass are in flight with the tile's vectors
        int32_t ty = 0;
        float ma = 0.f;
        if (t < m) {
            ty = in.type[base + t];
            ma = in.mass[base + t];
        }
        load_motion_tile(in, base, m, vec, sp, sv);
        __syncthreads();
        if (t < m) {
            const uint64_t i = base + t;
            x[i] = make_float4(sp[3 * t], sp[3 * t + 1], sp[3 * t + 2], ma);
            v[i] = make_float4(sv[3 * t], sv[3 * t + 1], sv[3 * t + 2], 0.f);
            type[i] = ty;
            obst += ty == FGB_TYPE_OBSTACLE;
        }
        __syncthreads();
    }
    for (int o = 16; o; o >>= 1) obst += __shfl_xor_sync(0xffffffffu, obst, o);
    if ((t & 31) == 0 && obst) atomicAdd(obstacles, obst);
}

__global__ void __launch_bounds__(kTile) k_pack_static(HostParticlesIn in, uint64_t n, uint32_t *__restrict__ col,
                                                      uint32_t *__restrict__ slot, uint64_t *__restrict__ ids) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        col[i] = in.colour ? in.colour[i] : 0xffffffffu;
        slot[i] = (uint32_t)i;
        ids[i] = in.id ? in.id[i] : i;
    }
}

// The fields of a download that are final once the step's grid is built (the
// particles' sorted order): type, colour, id, and mass (carried in p*.w).  Runs on a
// second stream while the step's gathers run; positions and velocities follow at
// the end of the step (k_unpack_to_host with only those two set).
__global__ void __launch_bounds__(kTile) k_unpack_static(HostParticlesOut out, uint64_t n,
                                                        const float4 *__restrict__ ps_grid,
                                                        const int32_t *__restrict__ type,
                                                        const uint32_t *__restrict__ col,
                                                        const uint32_t *__restrict__ slot,
                                                        const uint64_t *__restrict__ ids) {
    const uint64_t rs = out.stride;  // 0: packed arrays, else record i's fields i * stride further
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (out.mass) *(rs ? (float *)((char *)out.mass + i * rs) : out.mass + i) = ps_grid[i].w;
        if (out.type) *(rs ? (int32_t *)((char *)out.type + i * rs) : out.type + i) = type[i];
        if (out.colour) *(rs ? (uint32_t *)((char *)out.colour + i * rs) : out.colour + i) = col[i];
        if (out.id) {
            const uint32_t sl = slot[i];
            const uint64_t id = sl < n ? ids[sl] : sl;
            if (!rs) {
                out.id[i] = id;
            } else {  // records: 4-byte stores (a record's fields are 4-byte aligned)
                uint32_t *q = (uint32_t *)((char *)out.id + i * rs);
                q[0] = (uint32_t)id;
                if (out.id_bytes == 8) q[1] = (uint32_t)(id >> 32);
            }
        }
    }
}

// An upload from the caller's array of records: each CTA stages its tile of records
// in shared memory as 4-byte words read in order (every warp access a contiguous run
// of the host array), then each thread takes its particle's fields from there.
__global__ void __launch_bounds__(kTile) k_pack_records(HostRecords in, uint64_t n, float4 *__restrict__ x,
                                                       float4 *__restrict__ v, int32_t *__restrict__ type,
                                                       uint32_t *__restrict__ col, uint32_t *__restrict__ slot,
                                                       uint64_t *__restrict__ ids, uint32_t *__restrict__ obstacles) {
    __shared__ uint32_t sw[kTile * (kMaxRecordStride / 4)];
    const unsigned t = threadIdx.x;
    const uint32_t words = in.stride / 4;
    uint32_t obst = 0;
    for (uint64_t base = (uint64_t)blockIdx.x * kTile; base < n; base += (uint64_t)gridDim.x * kTile) {
        const uint32_t m = (uint32_t)(n - base < kTile ? n - base : kTile);
        const uint32_t *src = (const uint32_t *)(in.base + base * in.stride);
        for (uint32_t j = t; j < m * words; j += kTile) sw[j] = src[j];
        __syncthreads();
        if (t < m) {
            const uint64_t i = base + t;
            const uint32_t *r = sw + t * words;
            auto f32 = [&](int32_t off, int k) { return __uint_as_float(r[off / 4 + k]); };
            const float mass = in.off_mass >= 0 ? f32(in.off_mass, 0) : 0.f;
            const int32_t ty = in.off_type >= 0 ? (int32_t)r[in.off_type / 4] : FGB_TYPE_FLUID;
            x[i] = make_float4(f32(in.off_position, 0), f32(in.off_position, 1), f32(in.off_position, 2), mass);
            v[i] = make_float4(f32(in.off_velocity, 0), f32(in.off_velocity, 1), f32(in.off_velocity, 2), 0.f);
            type[i] = ty;
            col[i] = in.off_colour >= 0 ? r[in.off_colour / 4] : 0xffffffffu;
            slot[i] = (uint32_t)i;
            uint64_t id = i;
            if (in.off_id >= 0) {
                id = r[in.off_id / 4];
                if (in.id_bytes == 8) id |= (uint64_t)r[in.off_id / 4 + 1] << 32;
            }
            ids[i] = id;
            obst += ty == FGB_TYPE_OBSTACLE;
        }
        __syncthreads();
    }
    for (int o = 16; o; o >>= 1) obst += __shfl_xor_sync(0xffffffffu, obst, o);
    if ((t & 31) == 0 && obst) atomicAdd(obstacles, obst);
}

// A download into the caller's array of records, whole records at a time: each CTA
// builds its tile in shared memory (the described fields from the step's final state,
// every other byte zero) and stores it as 4-byte words in order, so every warp store
// covers a contiguous run of the host array.  Storing field by field instead leaves
// each warp store spread over 32 records, a few bytes in each.
__global__ void __launch_bounds__(kTile) k_unpack_records(HostRecords out, uint64_t n, const float4 *__restrict__ x,
                                                         const float4 *__restrict__ v, const int32_t *__restrict__ type,
                                                         const uint32_t *__restrict__ col,
                                                         const uint32_t *__restrict__ slot,
                                                         const uint64_t *__restrict__ ids) {
    __shared__ uint32_t sw[kTile * (kMaxRecordStride / 4)];
    const unsigned t = threadIdx.x;
    const uint32_t words = out.stride / 4;
    for (uint64_t base = (uint64_t)blockIdx.x * kTile; base < n; base += (uint64_t)gridDim.x * kTile) {
        const uint32_t m = (uint32_t)(n - base < kTile ? n - base : kTile);
        for (uint32_t j = t; j < m * words; j += kTile) sw[j] = 0u;
        __syncthreads();
        if (t < m) {
            const uint64_t i = base + t;
            uint32_t *r = sw + t * words;
            const float4 xi = x[i], vi = v[i];
            if (out.off_position >= 0) {
                uint32_t *q = r + out.off_position / 4;
                q[0] = __float_as_uint(xi.x);
                q[1] = __float_as_uint(xi.y);
                q[2] = __float_as_uint(xi.z);
            }
            if (out.off_velocity >= 0) {
                uint32_t *q = r + out.off_velocity / 4;
                q[0] = __float_as_uint(vi.x);
                q[1] = __float_as_uint(vi.y);
                q[2] = __float_as_uint(vi.z);
            }
            if (out.off_mass >= 0) r[out.off_mass / 4] = __float_as_uint(xi.w);
            if (out.off_type >= 0) r[out.off_type / 4] = (uint32_t)type[i];
            if (out.off_colour >= 0) r[out.off_colour / 4] = col[i];
            if (out.off_id >= 0) {
                const uint32_t sl = slot[i];
                const uint64_t id = sl < n ? ids[sl] : sl;
                r[out.off_id / 4] = (uint32_t)id;
                if (out.id_bytes == 8) r[out.off_id / 4 + 1] = (uint32_t)(id >> 32);
            }
        }
        __syncthreads();
        uint32_t *dst = (uint32_t *)(out.base + base * out.stride);
        for (uint32_t j = t; j < m * words; j += kTile) dst[j] = sw[j];
        __syncthreads();
    }
}

}  // namespace

void launch_unpack_records(const HostRecords &out, uint64_t n, const float4 *x, const float4 *v, const int32_t *type,
                           const uint32_t *col, const uint32_t *slot, const uint64_t *ids, cudaStream_t st) {
    if (n) k_unpack_records<<<grid_of(n), kTile, 0, st>>>(out, n, x, v, type, col, slot, ids);
}

void launch_pack_records(const HostRecords &in, uint64_t n, float4 *x, float4 *v, int32_t *type, uint32_t *col,
                         uint32_t *slot, uint64_t *ids, uint32_t *obstacles, cudaStream_t st) {
    if (n) k_pack_records<<<grid_of(n), kTile, 0, st>>>(in, n, x, v, type, col, slot, ids, obstacles);
}

HostParticlesOut record_fields(const HostRecords &r, bool motion, bool fixed) {
    auto at = [&](int32_t off) { return off >= 0 ? (void *)(r.base + off) : nullptr; };
    HostParticlesOut o{};
    if (motion) {
        o.position = (float *)at(r.off_position);
        o.velocity = (float *)at(r.off_velocity);
    }
    if (fixed) {
        o.mass = (float *)at(r.off_mass);
        o.type = (int32_t *)at(r.off_type);
        o.colour = (uint32_t *)at(r.off_colour);
        o.id = (uint64_t *)at(r.off_id);
    }
    o.stride = r.stride;
    o.id_bytes = r.id_bytes;
    return o;
}

void launch_unpack_static(const HostParticlesOut &out, uint64_t n, const float4 *ps_grid, const int32_t *type,
                          const uint32_t *col, const uint32_t *slot, const uint64_t *ids, cudaStream_t st) {
    // a quarter of the SMs: the stores only need to be in flight, and the gathers
    // that run beside them keep the rest
    unsigned g = (unsigned)std::min<uint64_t>((n + kTile - 1) / kTile, 38u * 2u);
    if (n) k_unpack_static<<<g ? g : 1u, kTile, 0, st>>>(out, n, ps_grid, type, col, slot, ids);
}

void launch_pack_motion(const HostParticlesIn &in, uint64_t n, float4 *x, float4 *v, int32_t *type,
                        uint32_t *obstacles, cudaStream_t st) {
    if (n) k_pack_motion<<<grid_of(n), kTile, 0, st>>>(in, n, x, v, type, obstacles);
}

void launch_pack_static(const HostParticlesIn &in, uint64_t n, uint32_t *col, uint32_t *slot, uint64_t *ids,
                        cudaStream_t st) {
    unsigned g = (unsigned)std::min<uint64_t>((n + kTile - 1) / kTile, 38u * 2u);
    if (n) k_pack_static<<<g ? g : 1u, kTile, 0, st>>>(in, n, col, slot, ids);
}

void launch_pack_from_host(const HostParticlesIn &in, uint64_t n, float4 *x, float4 *v, int32_t *type, uint32_t *col,
                           uint32_t *slot, uint64_t *ids, uint32_t *obstacles, cudaStream_t st) {
    if (n) k_pack_from_host<<<grid_of(n), kTile, 0, st>>>(in, n, x, v, type, col, slot, ids, obstacles);
}

void launch_unpack_to_host(const HostParticlesOut &out, uint64_t n, const float4 *x, const float4 *v,
                           const int32_t *type, const uint32_t *col, const uint32_t *slot, const uint64_t *ids,
                           cudaStream_t st) {
    if (n) k_unpack_to_host<<<grid_of(n), kTile, 0, st>>>(out, n, x, v, type, col, slot, ids);
}

}  // namespace fgb
