// sort.cu -- stable LSD radix sort of (key, value) u32 pairs, one sweep per digit.
//
// Replaces the reference's single-threaded std::sort of ~80-byte particle records by
// z-index (include/fluid/oclsph.hpp:733-743).  Unlike std::sort this sort is stable:
// particles of one cell keep their previous relative order, so the sorted order (and
// every sum over it) is a deterministic function of the input.
//
// Per pass (8-bit digit): each CTA takes the next tile id from an atomic counter,
// ranks its 4096 keys with warp-level match_any (in index order, hence stable),
// publishes its per-digit counts, looks back over earlier tiles' published counts
// (decoupled look-back) to find where its keys start, and scatters.  A pre-pass
// histograms all digits of all passes at once.  Every look-back wait is bounded.
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "fgb_device.cuh"
#include "fgb_internal.h"

namespace fgb {
namespace {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;
constexpr int kTile = kSortThreads * kSortItems;  // 4096 keys per tile
constexpr int kMaxPasses = 4;

constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagInclusive = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;

__global__ void __launch_bounds__(256) k_radix_histogram(const uint32_t *__restrict__ keys, uint32_t n,
                                                         int passes, uint32_t *__restrict__ hist) {
    __shared__ uint32_t sh[kMaxPasses][kRadix];
    for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&sh[p][(k >> (p * kRadixBits)) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) {
        uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Exclusive scan of each pass's 256 digit counts (one block per pass).
__global__ void __launch_bounds__(256) k_radix_offsets(const uint32_t *__restrict__ hist,
                                                       uint32_t *__restrict__ offsets) {
    __shared__ uint32_t warp_tot[kSortWarps];
    const int p = blockIdx.x, d = threadIdx.x, lane = d & 31, w = d >> 5;
    uint32_t v = hist[p * kRadix + d];
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    uint32_t base = 0;
    for (int i = 0; i < w; ++i) base += warp_tot[i];
    offsets[p * kRadix + d] = base + x - v;
}

__global__ void __launch_bounds__(kSortThreads) k_onesweep(
    const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
    uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, uint32_t n, int shift,
    const uint32_t *__restrict__ offsets, uint32_t *status, uint32_t *tile_counter, uint32_t *err,
    LookbackCtl ctl) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_hist[kSortWarps][kRadix + 1];
    __shared__ uint32_t s_base[kRadix + 1];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = tid; i < kSortWarps * (kRadix + 1); i += kSortThreads) (&s_hist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)kTile + (uint32_t)w * 32u * kSortItems;

    uint32_t k[kSortItems], v[kSortItems], rank[kSortItems];
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = base + (uint32_t)i * 32u + (uint32_t)lane;
        bool ok = idx < n;
        k[i] = ok ? keys_in[idx] : 0u;
        v[i] = ok ? vals_in[idx] : 0u;
    }
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = base + (uint32_t)i * 32u + (uint32_t)lane;
        uint32_t d = idx < n ? ((k[i] >> shift) & (kRadix - 1)) : (uint32_t)kRadix;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = s_hist[w][d];
        __syncwarp();
        rank[i] = before + __popc(peers & lt);
        if ((peers & lt) == 0) s_hist[w][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();

    // tid == digit: tile count and the exclusive prefix over warps
    {
        const uint32_t d = (uint32_t)tid;
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < kSortWarps; ++ww) {
            uint32_t c = s_hist[ww][d];
            s_hist[ww][d] = run;
            run += c;
        }
        uint32_t *my = status + (size_t)tile * kRadix + d;
        // a skipped tile (fgb_test_lookback_fault only) publishes nothing
        const bool publish = tile != ctl.skip_tile;
        uint32_t excl = 0;
        if (tile == 0) {
            if (publish) st_relaxed(my, kFlagInclusive | run);
        } else {
            if (publish) st_relaxed(my, kFlagAggregate | run);
            int t = (int)tile - 1;
            uint32_t spins = 0;
            while (t >= 0) {
                uint32_t s = ld_relaxed(status + (size_t)t * kRadix + d);
                if ((s & ~kValueMask) == 0) {
                    // a timed-out wait keeps the partial prefix: a sum over a subset of
                    // the earlier tiles' counts, so every scatter index stays below n
                    if (++spins > ctl.spin_limit) {
                        raise_error(err, ERR_SORT_LOOKBACK);
                        break;
                    }
                    continue;
                }
                excl += s & kValueMask;
                if (s & kFlagInclusive) break;
                --t;
            }
            if (publish) st_relaxed(my, kFlagInclusive | (excl + run));
        }
        s_base[d] = offsets[d] + excl;
    }
    __syncthreads();

#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = base + (uint32_t)i * 32u + (uint32_t)lane;
        if (idx < n) {
            uint32_t d = (k[i] >> shift) & (kRadix - 1);
            uint32_t pos = s_base[d] + s_hist[w][d] + rank[i];
            if (pos < n) {  // only a timed-out look-back can produce pos >= n
                keys_out[pos] = k[i];
                vals_out[pos] = v[i];
            } else {
                raise_error(err, ERR_SORT_LOOKBACK);
            }
        }
    }
}

struct SortLayout {
    size_t hist, offsets, counters, status, alt_keys, alt_vals, total;
    uint32_t tiles;
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

SortLayout sort_layout(uint64_t n) {
    SortLayout L;
    L.tiles = (uint32_t)((n + kTile - 1) / kTile);
    size_t o = 0;
    L.hist = o;
    o = align256(o + sizeof(uint32_t) * kMaxPasses * kRadix);
    L.offsets = o;
    o = align256(o + sizeof(uint32_t) * kMaxPasses * kRadix);
    L.counters = o;
    o = align256(o + sizeof(uint32_t) * kMaxPasses);
    L.status = o;
    o = align256(o + sizeof(uint32_t) * (size_t)kMaxPasses * (L.tiles ? L.tiles : 1) * kRadix);
    L.alt_keys = o;
    o = align256(o + sizeof(uint32_t) * (n ? n : 1));
    L.alt_vals = o;
    o = align256(o + sizeof(uint32_t) * (n ? n : 1));
    L.total = o;
    return L;
}

}  // namespace

namespace {
std::atomic<uint64_t> g_lookback{(uint64_t)kSpinLimit << 32 | 0xffffffffull};
}  // namespace

LookbackCtl lookback_ctl() {
    const uint64_t v = g_lookback.load(std::memory_order_relaxed);
    return LookbackCtl{(uint32_t)v, (uint32_t)(v >> 32)};
}

uint64_t radix_scratch_bytes(uint64_t n) { return sort_layout(n).total; }

int radix_passes(uint32_t key_bits) {
    int p = (int)((key_bits + kRadixBits - 1) / kRadixBits);
    return p < 1 ? 1 : p;
}

cudaError_t radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                             uint32_t *vals_out, uint64_t n, uint32_t key_bits, void *scratch,
                             uint64_t scratch_bytes, cudaStream_t stream, uint32_t *err,
                             uint64_t *launches) {
    if (n == 0) return cudaSuccess;
    if (key_bits > 32 || n > (uint64_t)kValueMask) return cudaErrorInvalidValue;
    SortLayout L = sort_layout(n);
    if (scratch_bytes < L.total || scratch == nullptr) return cudaErrorInvalidValue;
    char *s = (char *)scratch;
    uint32_t *hist = (uint32_t *)(s + L.hist);
    uint32_t *offsets = (uint32_t *)(s + L.offsets);
    uint32_t *counters = (uint32_t *)(s + L.counters);
    uint32_t *status = (uint32_t *)(s + L.status);
    uint32_t *alt_k = (uint32_t *)(s + L.alt_keys);
    uint32_t *alt_v = (uint32_t *)(s + L.alt_vals);
    const int passes = radix_passes(key_bits);
    const LookbackCtl ctl = lookback_ctl();
    // hist, offsets, counters and the status words of every pass start at zero
    cudaError_t e = cudaMemsetAsync(s, 0, L.alt_keys, stream);
    if (e != cudaSuccess) return e;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 1216) blocks = 1216;
    k_radix_histogram<<<blocks, 256, 0, stream>>>(keys_in, (uint32_t)n, passes, hist);
    k_radix_offsets<<<passes, 256, 0, stream>>>(hist, offsets);
    const uint32_t *src_k = keys_in, *src_v = vals_in;
    for (int p = 0; p < passes; ++p) {
        bool to_out = ((passes - 1 - p) % 2) == 0;
        uint32_t *dk = to_out ? keys_out : alt_k;
        uint32_t *dv = to_out ? vals_out : alt_v;
        k_onesweep<<<L.tiles, kSortThreads, 0, stream>>>(
            src_k, src_v, dk, dv, (uint32_t)n, p * kRadixBits, offsets + p * kRadix,
            status + (size_t)p * L.tiles * kRadix, counters + p, err, ctl);
        src_k = dk;
        src_v = dv;
    }
    if (launches) *launches += 2 + passes;
    return cudaGetLastError();
}

}  // namespace fgb

extern "C" {

uint64_t fgb_radix_sort_scratch_bytes(uint64_t n) {
    // one extra u32 at the end holds the device error flag of the standalone call
    return fgb::radix_scratch_bytes(n) + 256;
}

int fgb_radix_sort_pairs_u32(const uint32_t *d_keys_in, const uint32_t *d_vals_in, uint32_t *d_keys_out,
                             uint32_t *d_vals_out, uint64_t n, uint32_t key_bits, void *d_scratch,
                             uint64_t scratch_bytes, void *cuda_stream) {
    if (n && (!d_keys_in || !d_vals_in || !d_keys_out || !d_vals_out))
        return fgb::fail(FGB_ERR_INVALID, "radix sort: null pointer");
    if (key_bits == 0 || key_bits > 32) return fgb::fail(FGB_ERR_INVALID, "radix sort: key_bits must be 1..32");
    if (scratch_bytes < fgb_radix_sort_scratch_bytes(n))
        return fgb::fail(FGB_ERR_INVALID, "radix sort: scratch smaller than fgb_radix_sort_scratch_bytes(n)");
    uint64_t core = fgb::radix_scratch_bytes(n);
    uint32_t *err = (uint32_t *)((char *)d_scratch + core);
    cudaStream_t st = (cudaStream_t)cuda_stream;
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess)
        e = fgb::radix_sort_pairs(d_keys_in, d_vals_in, d_keys_out, d_vals_out, n, key_bits, d_scratch, core, st,
                                  err, nullptr);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "radix sort");
    return FGB_OK;
}

int fgb_radix_sort_error(const void *d_scratch, uint64_t n, void *cuda_stream, uint32_t *flags) {
    if (!d_scratch || !flags) return fgb::fail(FGB_ERR_INVALID, "radix sort error: null argument");
    return fgb::read_clear_flag((char *)d_scratch + fgb::radix_scratch_bytes(n), (cudaStream_t)cuda_stream, flags,
                                "radix sort error");
}

int fgb_test_lookback_fault(uint32_t skip_tile, uint32_t spin_limit) {
    if (skip_tile != 0xffffffffu && spin_limit == 0)
        return fgb::fail(FGB_ERR_INVALID, "lookback fault: a skipped tile needs a spin limit above 0");
    if (skip_tile == 0xffffffffu) spin_limit = fgb::kSpinLimit;
    fgb::g_lookback.store((uint64_t)spin_limit << 32 | skip_tile, std::memory_order_relaxed);
    return FGB_OK;
}
}
