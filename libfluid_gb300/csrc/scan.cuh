// scan.cuh -- single-pass exclusive prefix sum with decoupled look-back.
//
// Replaces the reference's per-work-group tree reduction of marching-cubes triangle
// counts followed by a blocking host-side sum (include/fluid/oclsph_kernel.h:545-596,
// include/fluid/oclsph.hpp:450-465): here the counts become exclusive offsets on the
// device in one pass, so triangles can be written at fixed, deterministic positions.
//
// The input is produced by a loader functor (`uint32_t operator()(uint64_t i)`, or a
// `run` over a thread's consecutive items), so
// the marching-cubes case classification is fused into the scan's load.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>
#include <cuda_runtime.h>

#include "fgb_device.cuh"

namespace fgb {

// Look-back settings of the next launches (sort.cu; fgb_test_lookback_fault).
LookbackCtl lookback_ctl();

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

// A loader may also offer `run(first, n, v)`, filling v[0..kScanItems) with the items
// first, first + 1, ... (0 at and past n) in one call, when consecutive items share work.
template <class L, class = void>
struct kLoadsRuns : std::false_type {};
template <class L>
struct kLoadsRuns<L, std::void_t<decltype(std::declval<const L &>().run(
                         uint64_t{}, uint64_t{}, std::declval<uint32_t (&)[kScanItems]>()))>> : std::true_type {};

constexpr unsigned long long kScanAggregate = 1ull << 32;
constexpr unsigned long long kScanInclusive = 2ull << 32;

template <class Load>
__global__ void __launch_bounds__(kScanThreads)
    k_scan(Load load, uint32_t *__restrict__ out, uint64_t n, unsigned long long *status,
           uint32_t *tile_counter, uint32_t *total, uint32_t *err, LookbackCtl ctl) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kScanThreads / 32];
    __shared__ uint32_t s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t first = (uint64_t)tile * kScanTile + (uint64_t)tid * kScanItems;

    uint32_t v[kScanItems];
    uint32_t sum = 0;
    if constexpr (kLoadsRuns<Load>::value) {
        load.run(first, n, v);
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) {
            uint64_t idx = first + i;
            v[i] = idx < n ? load(idx) : 0u;
        }
    }
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) sum += v[i];
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    uint32_t warp_base = 0, block_total = 0;
#pragma unroll
    for (int i = 0; i < kScanThreads / 32; ++i) {
        uint32_t t = s_warp[i];
        if (i < w) warp_base += t;
        block_total += t;
    }
    if (tid == 0) {
        unsigned long long *my = status + tile;
        // a skipped tile (fgb_test_lookback_fault only) publishes nothing
        const bool publish = tile != ctl.skip_tile;
        uint32_t prefix = 0;
        if (tile == 0) {
            if (publish) st_relaxed64(my, kScanInclusive | block_total);
        } else {
            if (publish) st_relaxed64(my, kScanAggregate | block_total);
            int t = (int)tile - 1;
            uint32_t spins = 0;
            while (t >= 0) {
                unsigned long long s = ld_relaxed64(status + t);
                if ((s >> 32) == 0) {
                    // the wait gives up with a partial prefix; outputs are then wrong
                    // but every store stays at its own index below n
                    if (++spins > ctl.spin_limit) {
                        raise_error(err, ERR_SCAN_LOOKBACK);
                        break;
                    }
                    continue;
                }
                prefix += (uint32_t)(s & 0xffffffffull);
                if (s & kScanInclusive) break;
                --t;
            }
            if (publish) st_relaxed64(my, kScanInclusive | (unsigned long long)(uint32_t)(prefix + block_total));
        }
        s_prefix = prefix;
        uint64_t tiles = (n + kScanTile - 1) / kScanTile;
        if (total && (uint64_t)tile + 1 == tiles) *total = prefix + block_total;
    }
    __syncthreads();
    uint32_t run = s_prefix + warp_base + (x - sum);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        uint64_t idx = first + i;
        if (idx < n) out[idx] = run;
        run += v[i];
    }
}

inline uint64_t scan_tiles(uint64_t n) { return (n + kScanTile - 1) / kScanTile; }

// Scratch: [status u64 per tile][tile counter u32] (zeroed before each scan).
inline uint64_t scan_scratch(uint64_t n) {
    return ((scan_tiles(n) ? scan_tiles(n) : 1) * sizeof(unsigned long long) + 256 + 255) & ~uint64_t(255);
}

template <class Load>
cudaError_t scan_launch(Load load, uint32_t *out, uint32_t *total, uint64_t n, void *scratch,
                        uint64_t scratch_bytes, cudaStream_t stream, uint32_t *err, uint64_t *launches) {
    if (n == 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), stream);
        return cudaSuccess;
    }
    if (scratch_bytes < scan_scratch(n)) return cudaErrorInvalidValue;
    uint64_t tiles = scan_tiles(n);
    unsigned long long *status = (unsigned long long *)scratch;
    uint32_t *counter = (uint32_t *)((char *)scratch + tiles * sizeof(unsigned long long));
    cudaError_t e = cudaMemsetAsync(scratch, 0, tiles * sizeof(unsigned long long) + sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    k_scan<Load><<<(unsigned)tiles, kScanThreads, 0, stream>>>(load, out, n, status, counter, total, err,
                                                               lookback_ctl());
    if (launches) *launches += 1;
    return cudaGetLastError();
}

struct LoadU32 {
    const uint32_t *p;
    __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return __ldg(p + i); }
};

}  // namespace fgb
