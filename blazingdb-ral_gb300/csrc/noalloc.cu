// noalloc.cu — apply_boolean_mask without any device allocation.
//
// Some callers cannot allocate device memory during a query: engines whose
// memory pool has already reserved the whole GPU (a second allocator would
// fail or fragment it), and latency-critical paths that must never enter the
// driver's allocator.  ral_apply_boolean_mask needs a small scratch block for
// the single-pass compaction's tile states; this variant takes that block from
// a fixed array compiled into the library instead of allocating it.
//
// The array lives in every device's memory as soon as the library's module is
// loaded there and stays until the process exits.  Its host-side name is only a
// stand-in for the symbol: each call looks up the array's device address on the
// current device with cudaGetSymbolAddress and passes it to the kernel.  (The
// address is not cached: after a cudaDeviceReset the module is loaded again and
// the array may move.)  All calls share the one array: it is cleared before each
// use, and calls whose GPU work overlaps (two threads, or two streams, at once)
// race on it.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "engine.h"
#include "kernels.h"
#include "ral/ral_c.h"

namespace {

constexpr size_t kScratchBytes = 256 * 1024;
constexpr int64_t kScratchWords = (int64_t)(kScratchBytes / sizeof(unsigned long long));
// Largest stencil the array can serve: 3 header words, then one status word per 4096-row tile.
constexpr int64_t kMaxRows = (kScratchWords - 3) * ral::kCompactTileRows;
static_assert(RAL_NOALLOC_MAX_ROWS == kMaxRows, "ral_c.h states a different limit");

static __device__ __align__(256) unsigned long long g_scratch[kScratchWords];

// Device address of g_scratch on the current device.  The first lookup on a device loads the
// library's module there.
int scratch_on_current_device(unsigned long long** out) {
    void* p = nullptr;
    if (int e = ral::check_cuda(cudaGetSymbolAddress(&p, g_scratch), "cudaGetSymbolAddress")) return e;
    *out = static_cast<unsigned long long*>(p);
    return ral::kSuccess;
}

}  // namespace

extern "C" int ral_apply_boolean_mask_noalloc(const gdf_column* stencil, gdf_column* out_indices,
                                              gdf_size_type* num_rows_out) {
    try {
        using namespace ral;
        if (!stencil || !out_indices || !num_rows_out) return set_error(kInvalidArgument, "null argument");
        if (gdf_dtype_size(stencil->dtype) != 1) return set_error(kInvalidArgument, "stencil must be INT8 or BOOL8");
        if (out_indices->dtype != GDF_INT32) return set_error(kInvalidArgument, "out_indices must be INT32");
        if (stencil->valid && ((uintptr_t)stencil->valid & 3)) return set_error(kInvalidArgument, "mask must be 4-byte aligned");
        const int64_t n = stencil->size;
        if (n < 0) return set_error(kInvalidArgument, "negative row count");
        if (n > kMaxRows)
            return set_error(kInvalidArgument, "ral_apply_boolean_mask_noalloc: " + std::to_string(n) +
                                                   " rows exceed the fixed scratch limit of " + std::to_string(kMaxRows) +
                                                   " rows; use ral_apply_boolean_mask");
        unsigned long long* scratch = nullptr;
        if (int e = scratch_on_current_device(&scratch)) return e;
        if (n == 0) {
            out_indices->size = 0;
            *num_rows_out = 0;
            return kSuccess;
        }
        if (!stencil->data || !out_indices->data) return set_error(kInvalidArgument, "column without data");
        cudaStream_t st = cudaStreamPerThread;
        const int64_t words = compact_scratch_words(n);
        if (int e = check_cuda(cudaMemsetAsync(scratch, 0, (size_t)words * 8, st), "cudaMemsetAsync")) return e;
        if (int e = check_cuda(launch_compact_stencil((const int8_t*)stencil->data, (const uint32_t*)stencil->valid, n,
                                                      (int32_t*)out_indices->data, scratch, st),
                               "compaction"))
            return e;
        unsigned long long h[3] = {0, 0, 0};
        if (int e = check_cuda(cudaMemcpyAsync(h, scratch, sizeof h, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync"))
            return e;
        if (int e = check_cuda(cudaStreamSynchronize(st), "apply_boolean_mask_noalloc")) return e;
        if (h[1]) return set_error(kTimeout, "compaction look-back wait gave up");
        out_indices->size = (gdf_size_type)h[2];
        *num_rows_out = (gdf_size_type)h[2];
        return kSuccess;
    } catch (const std::exception& e) {
        return ral::set_error(ral::kInvalidArgument, e.what());
    }
}
