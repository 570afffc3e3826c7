// scan.cu -- the u32 instantiation of the single-pass scan and its C ABI entries.
#include <mutex>

#include "fgb_internal.h"
#include "scan.cuh"

namespace fgb {

uint64_t scan_u32_scratch_bytes(uint64_t n) { return scan_scratch(n); }

cudaError_t scan_u32(const uint32_t *in, uint32_t *out, uint32_t *total, uint64_t n, void *scratch,
                     uint64_t scratch_bytes, cudaStream_t stream, uint32_t *err, uint64_t *launches) {
    return scan_launch(LoadU32{in}, out, total, n, scratch, scratch_bytes, stream, err, launches);
}

}  // namespace fgb

extern "C" {

uint64_t fgb_scan_scratch_bytes(uint64_t n) { return fgb::scan_scratch(n) + 256; }

int fgb_exclusive_scan_u32(const uint32_t *d_in, uint32_t *d_out, uint32_t *d_total, uint64_t n, void *d_scratch,
                           uint64_t scratch_bytes, void *cuda_stream) {
    if (n && (!d_in || !d_out)) return fgb::fail(FGB_ERR_INVALID, "scan: null pointer");
    if (n > 0xffffffffull) return fgb::fail(FGB_ERR_CAPACITY, "scan: n above 2^32-1");
    if (scratch_bytes < fgb_scan_scratch_bytes(n))
        return fgb::fail(FGB_ERR_INVALID, "scan: scratch smaller than fgb_scan_scratch_bytes(n)");
    uint64_t core = fgb::scan_scratch(n);
    uint32_t *err = (uint32_t *)((char *)d_scratch + core);
    cudaStream_t st = (cudaStream_t)cuda_stream;
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = fgb::scan_u32(d_in, d_out, d_total, n, d_scratch, core, st, err, nullptr);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "scan");
    return FGB_OK;
}
}

// ---------------------------------------------------------------------------
// Scan without any allocation, for callers that cannot call cudaMalloc: a host
// whose memory manager owns every device allocation, a plugin host that forbids
// its plugins to allocate, or a real-time loop where an allocation could block or
// fail.  Its look-back scratch (one status word per tile, the
// tile counter and an error flag) lives in the file-scope device array below,
// sized for at most FGB_SCAN_NOALLOC_MAX_N elements; every GPU that loads the
// library holds this array until the process exits.
namespace {

constexpr uint64_t kNoAllocTiles = FGB_SCAN_NOALLOC_MAX_N / fgb::kScanTile;
constexpr uint64_t kNoAllocCore = kNoAllocTiles * sizeof(unsigned long long) + 256;
constexpr uint64_t kNoAllocBytes = kNoAllocCore + 256;  // + the error flag
static_assert(FGB_SCAN_NOALLOC_MAX_N % fgb::kScanTile == 0, "whole tiles");
static_assert(kNoAllocCore >= 0, "layout");

static __device__ __align__(256) unsigned char g_scan_noalloc_scratch[kNoAllocBytes];

// Device address of the array, looked up once per device.  In host code the name
// g_scan_noalloc_scratch is only a stand-in for the symbol, never a device address.
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

int noalloc_scratch(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "scan_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fgb::fail(FGB_ERR_UNSUPPORTED, "scan_noalloc: device ordinal >= 64");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_scan_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return fgb::fail_cuda(e, "scan_noalloc: cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = ptr;
    }
    *out = g_noalloc_ptr[dev];
    return FGB_OK;
}

}  // namespace

extern "C" int fgb_exclusive_scan_u32_noalloc(const uint32_t *d_in, uint32_t *d_out, uint32_t *d_total, uint64_t n,
                                              void *cuda_stream) {
    if (n && (!d_in || !d_out)) return fgb::fail(FGB_ERR_INVALID, "scan_noalloc: null pointer");
    if (n > FGB_SCAN_NOALLOC_MAX_N)
        return fgb::fail(FGB_ERR_CAPACITY, "scan_noalloc: n exceeds FGB_SCAN_NOALLOC_MAX_N (16777216); "
                                           "use fgb_exclusive_scan_u32 with caller scratch");
    void *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc != FGB_OK) return rc;
    uint32_t *err = (uint32_t *)((char *)scratch + kNoAllocCore);
    cudaStream_t st = (cudaStream_t)cuda_stream;
    // the array keeps the previous call's contents: the flag, the status words and
    // the tile counter must start at zero (scan_launch clears the latter two)
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = fgb::scan_u32(d_in, d_out, d_total, n, scratch, kNoAllocCore, st, err, nullptr);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "scan_noalloc");
    return FGB_OK;
}
