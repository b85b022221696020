// engine.h — host side of the expression path: program -> kernel -> launch.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "codegen.h"
#include "jit.h"
#include "program.h"
#include "ral/gdf_compat.h"

namespace ral {

// Status codes of the C ABI (include/ral/ral_c.h).
enum Status : int {
    kSuccess = 0,
    kInvalidArgument = 1,
    kUnsupported = 2,
    kCudaError = 3,
    kJitError = 4,
    kAllocError = 5,
    kTimeout = 6,
    kParseError = 7,
};

// Thread-local error text of the last failing call.
int set_error(int code, const std::string& msg);
const char* last_error();

// Maps a CUDA error to kCudaError with context; returns kSuccess on cudaSuccess.
int check_cuda(cudaError_t e, const char* what);

struct ProgramArrays {
    const int16_t* left;
    const int16_t* right;
    const int16_t* outs;
    int32_t n_ops;
    const int16_t* final_positions;
    const int32_t* bops;
    const int32_t* uops;
    const gdf_scalar* lscalars;
    const gdf_scalar* rscalars;
};

// Launch shape of a perform_operation kernel: the default, with RAL_EVAL_TUNE's overrides.
Shape eval_shape(const Program& p);

struct EvalOptions {
    cudaStream_t stream = nullptr;
    bool sync = true;
    // when non-null, receives per output the number of null rows in [0, n)
    // (outputs without a valid mask report 0)
    int64_t* null_counts = nullptr;
    // override the default launch shape (autotuner); G == 0 keeps the default
    Shape shape{0, 0, 0, 0};
    // treat every input's validity mask as possibly holding nulls, ignoring
    // null_count (fused filter+project semantics)
    bool ignore_null_count = false;
    // when non-null (and null_counts is null): device array the kernel adds each output's
    // number of valid rows to, without any synchronisation; the caller zeroes and reads it
    uint64_t* device_valid_counts = nullptr;
};

// perform_operation over columns in host memory: the rows stream through the GPU in chunks of
// chunk_rows (0: the default), each chunk's host-to-device copies, kernel and device-to-host copies
// on one of three streams, so that copies in both directions overlap each other and the kernels.
// Results and null counts are those of perform_operation over the whole columns; host buffers
// should be page-locked for the copies to overlap.
int perform_operation_host(gdf_column* const* outputs, int n_out, gdf_column* const* inputs, int n_in,
                           const ProgramArrays& pa, int64_t chunk_rows);

// perform_operation over gdf_columns.  Outputs are written in place.
int perform_operation(gdf_column* const* outputs, int n_out, gdf_column* const* inputs, int n_in,
                      const ProgramArrays& prog, const EvalOptions& opt);

// Build a Program from gdf_columns (shared by the eval, filter and batch paths).
int build_program(Program& p, gdf_column* const* outputs, int n_out, gdf_column* const* inputs, int n_in,
                  const ProgramArrays& prog, bool ignore_null_count);

// Number of SMs and resident blocks per SM for a compiled kernel on the current device.
int launch_blocks(const CompiledKernel& k, int threads, int64_t work_items_per_block_unit, int64_t units);
// SMs of the current device; resident blocks per SM of a compiled kernel (cached per device).
int device_sms();
int blocks_per_sm(const CompiledKernel& k, int threads);
// Freed stream-ordered allocations of the current device stay in its default pool instead of going
// back to the driver at each synchronisation, so the large per-call buffers of the scans and the
// server are reused rather than mapped again (set once per device for the process).
void keep_pool_memory();

// The copy stream of the calling thread on the current device, with its events (made once, kept
// for the thread's life): host-to-device copies issued on it overlap kernels on the caller's stream.
struct CopyLane {
    cudaStream_t s = nullptr;
    cudaEvent_t ready = nullptr;
    std::vector<cudaEvent_t> events;  // grown on demand by lane_event
};
int copy_lane(CopyLane*& out);
// The lane's k-th event (created on first use).
int lane_event(CopyLane& lane, size_t k, cudaEvent_t* ev);
// On every exit of its scope: the calling stream waits for the copies issued on the lane so far,
// so buffers freed on the calling stream afterwards are no longer being written.
struct LaneJoin {
    CopyLane* lane;
    cudaStream_t st;
    ~LaneJoin() {
        cudaEventRecord(lane->ready, lane->s);
        cudaStreamWaitEvent(st, lane->ready, 0);
    }
};

// Parameter block filled in ParamLayout order.
void fill_scalars(const Program& p, const ParamLayout& L, std::vector<uint64_t>& slots);

// ---- per-call timing of the synchronous filter entry points ----------------------------------
// Off unless enabled (RAL_CALL_TIMING=1 or ral_debug_call_timing): each call adds its host
// preparation (entry to the first enqueue), its enqueue (memsets, launch, copy back), its wait
// for completion and the device time of its kernel (CUDA events around the launch), in
// microseconds.
bool call_timing_enabled();
void call_timing_start();                       // at the entry point
void call_timing_mark_prepared();               // before the first enqueue
void call_timing_add(double enqueue_us, double wait_us, double device_us);  // after the sync
int call_timing_query(bool enable, bool reset, int64_t* calls, double* us4);

// process_aggregate without GROUP BY, expressions fused with the reduction (aggregate.cpp).
int process_aggregate(gdf_column* const* frame, int n_cols, const char* query, gdf_scalar* results, int capacity,
                      int* num_results, cudaStream_t st);
// Generated source (and optionally an NVRTC compile) of a plan's aggregate kernel.
int aggregate_source(const gdf_dtype* dtypes, const int32_t* nullable, const int64_t* null_counts, int n_cols,
                     const char* query, bool compile, std::string& source, std::string& log);

// Count of kernels this library has launched (all entry points).
void note_launch(int count = 1);
long long launch_count();

// Process-wide options.
struct Config {
    bool float_literal_compat = false;  // RAL_FLOAT_LITERAL_COMPAT=1
};
Config& config();

}  // namespace ral
