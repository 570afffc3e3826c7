// scan.cu -- the u32 instantiation of the single-pass scan and its C ABI entry.
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
