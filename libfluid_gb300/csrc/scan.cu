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

int read_clear_flag(void *d_flag, cudaStream_t stream, uint32_t *flags, const char *where) {
    cudaError_t e = cudaMemcpyAsync(flags, d_flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flag, 0, sizeof(uint32_t), stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail_cuda(e, where);
    return FGB_OK;
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

int fgb_scan_error(const void *d_scratch, uint64_t n, void *cuda_stream, uint32_t *flags) {
    if (!d_scratch || !flags) return fgb::fail(FGB_ERR_INVALID, "scan error: null argument");
    return fgb::read_clear_flag((char *)d_scratch + fgb::scan_scratch(n), (cudaStream_t)cuda_stream, flags,
                                "scan error");
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

// Device address of the array per device.  In host code the name
// g_scan_noalloc_scratch is only a stand-in for the symbol, never a device address.
// The address is looked up again on every call made outside a stream capture (the
// lookup is cheap once the module is loaded, and a cudaDeviceReset reloads the module
// at a new address); a call being captured uses the address of the last call made
// outside a capture, so the first call on a device must precede any capture.
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

int noalloc_scratch(cudaStream_t st, void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "scan_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fgb::fail(FGB_ERR_UNSUPPORTED, "scan_noalloc: device ordinal >= 64");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "scan_noalloc: cudaStreamIsCapturing");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_scan_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return fgb::fail_cuda(e, "scan_noalloc: cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = ptr;
    } else if (!g_noalloc_ptr[dev]) {
        return fgb::fail(FGB_ERR_INVALID, "scan_noalloc: the first call on a device must precede any stream capture");
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
    cudaStream_t st = (cudaStream_t)cuda_stream;
    void *scratch = nullptr;
    int rc = noalloc_scratch(st, &scratch);
    if (rc != FGB_OK) return rc;
    uint32_t *err = (uint32_t *)((char *)scratch + kNoAllocCore);
    // the array keeps the previous call's contents: the status words and the tile
    // counter must start at zero (scan_launch clears them); the error flag gathers the
    // calls since the last fgb_scan_noalloc_error, which clears it (zero at load)
    cudaError_t e = fgb::scan_u32(d_in, d_out, d_total, n, scratch, kNoAllocCore, st, err, nullptr);
    if (e != cudaSuccess) return fgb::fail_cuda(e, "scan_noalloc");
    return FGB_OK;
}

extern "C" int fgb_scan_noalloc_error(void *cuda_stream, uint32_t *flags) {
    if (!flags) return fgb::fail(FGB_ERR_INVALID, "scan_noalloc error: null argument");
    cudaStream_t st = (cudaStream_t)cuda_stream;
    void *scratch = nullptr;
    int rc = noalloc_scratch(st, &scratch);
    if (rc != FGB_OK) return rc;
    return fgb::read_clear_flag((char *)scratch + kNoAllocCore, st, flags, "scan_noalloc error");
}
