// filter.cpp — LogicalFilter: stencil, compaction and gather of every column.
//
// Reference flow (src/CalciteInterpreter.cpp:509-573): evaluate the condition
// into an INT8 stencil with a validity mask, build an int32 iota, compact it
// with cudf::apply_boolean_mask (row kept when the stencil bit is valid and
// the byte is nonzero), then materialize_column every frame column.
#include "filter.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "codegen.h"
#include "engine.h"
#include "frontend.h"
#include "jit.h"
#include "kernels.h"

namespace ral {

namespace {

struct DeviceBuffer {
    void* p = nullptr;
    cudaStream_t st = nullptr;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() {
        if (p) cudaFreeAsync(p, st);
    }
    int alloc(size_t bytes, cudaStream_t s) {
        st = s;
        if (bytes == 0) bytes = 8;
        return check_cuda(cudaMallocAsync(&p, bytes, s), "cudaMallocAsync");
    }
};

int check_outputs(gdf_column* const* frame, int ncols, gdf_column* const* outs) {
    for (int c = 0; c < ncols; c++) {
        if (!frame[c] || !outs[c]) return set_error(kInvalidArgument, "null column");
        if (outs[c]->dtype != frame[c]->dtype) return set_error(kInvalidArgument, "out column dtype differs from the frame's");
        if ((frame[c]->valid != nullptr) != (outs[c]->valid != nullptr))
            return set_error(kInvalidArgument, "out column must carry a validity buffer exactly when the frame column does");
        if (frame[c]->size > 0 && !outs[c]->data) return set_error(kInvalidArgument, "out column without data");
        if (gdf_dtype_size(frame[c]->dtype) == 0) return set_error(kUnsupported, "column dtype has no fixed width");
        if (frame[c]->size != frame[0]->size) return set_error(kInvalidArgument, "frame columns differ in size");
    }
    return kSuccess;
}

int filter_mode(const FilterOptions& opt) {
    if (opt.mode >= 0) return opt.mode;
    const char* m = std::getenv("RAL_FILTER_MODE");
    if (m && std::string(m) == "unfused") return 1;
    return 0;
}

// The stencil of the condition: either a frame column ("$k") or a program output.
struct Stencil {
    const int8_t* data = nullptr;
    const uint32_t* valid = nullptr;
    DeviceBuffer data_buf, valid_buf;
};

int make_stencil(gdf_column* const* frame, int ncols, const std::string& cond, Stencil& s, cudaStream_t st) {
    ExpressionPlan ep = plan_expression(cond, ncols);
    const int64_t n = frame[0]->size;
    if (ep.clone) {
        const gdf_column* c = frame[ep.clone_column];
        if (gdf_dtype_size(c->dtype) != 1)
            return set_error(kUnsupported, "a bare \"$k\" condition needs a one-byte column (the stencil is read as BOOL8)");
        s.data = (const int8_t*)c->data;
        s.valid = (const uint32_t*)c->valid;
        return kSuccess;
    }
    if (int e = s.data_buf.alloc((size_t)n, st)) return e;
    if (int e = s.valid_buf.alloc(gdf_valid_allocation_size(n), st)) return e;
    gdf_column col{};
    col.data = s.data_buf.p;
    col.valid = (gdf_valid_type*)s.valid_buf.p;
    col.size = (gdf_size_type)n;
    col.dtype = GDF_INT8;
    gdf_column* outs[1] = {&col};
    std::vector<gdf_column*> ins;
    for (int c : ep.input_columns) ins.push_back(frame[c]);
    ProgramArrays pa{ep.pv.left.data(), ep.pv.right.data(), ep.pv.outs.data(), (int32_t)ep.pv.left.size(),
                     ep.pv.final_pos.data(), ep.pv.bops.data(), ep.pv.uops.data(), ep.pv.lscalars.data(),
                     ep.pv.rscalars.data()};
    EvalOptions eo;
    eo.stream = st;
    eo.sync = false;
    if (int e = perform_operation(outs, 1, ins.data(), (int)ins.size(), pa, eo)) return e;
    s.data = (const int8_t*)s.data_buf.p;
    s.valid = (const uint32_t*)s.valid_buf.p;
    return kSuccess;
}

// stencil -> row indices (count on the host)
int compact(const Stencil& s, int64_t n, DeviceBuffer& idx, int64_t& n_out, cudaStream_t st) {
    if (int e = idx.alloc((size_t)n * 4, st)) return e;
    DeviceBuffer scratch;
    const int64_t words = compact_scratch_words(n);
    if (int e = scratch.alloc((size_t)words * 8, st)) return e;
    cudaMemsetAsync(scratch.p, 0, (size_t)words * 8, st);
    if (int e = check_cuda(launch_compact_stencil(s.data, s.valid, n, (int32_t*)idx.p, (unsigned long long*)scratch.p, st),
                           "compaction"))
        return e;
    unsigned long long h[3] = {0, 0, 0};
    cudaMemcpyAsync(h, scratch.p, sizeof h, cudaMemcpyDeviceToHost, st);
    if (int e = check_cuda(cudaStreamSynchronize(st), "compaction")) return e;
    if (h[1]) return set_error(kTimeout, "compaction look-back wait gave up");
    n_out = (int64_t)h[2];
    return kSuccess;
}

int gather_all(gdf_column* const* frame, int ncols, const int32_t* idx, int64_t n_out, gdf_column* const* outs,
               cudaStream_t st) {
    DeviceBuffer counts;
    if (int e = counts.alloc(sizeof(unsigned long long) * ncols, st)) return e;
    cudaMemsetAsync(counts.p, 0, sizeof(unsigned long long) * ncols, st);
    unsigned long long* dc = (unsigned long long*)counts.p;
    for (int c = 0; c < ncols; c++) {
        if (int e = check_cuda(launch_gather(gdf_dtype_size(frame[c]->dtype), frame[c]->data,
                                             (const uint32_t*)frame[c]->valid, frame[c]->size, idx, 4, n_out,
                                             outs[c]->data,
                                             (uint32_t*)outs[c]->valid, outs[c]->valid ? dc + c : nullptr, st),
                               "gather"))
            return e;
    }
    std::vector<unsigned long long> h(ncols, 0);
    cudaMemcpyAsync(h.data(), dc, sizeof(unsigned long long) * ncols, cudaMemcpyDeviceToHost, st);
    if (int e = check_cuda(cudaStreamSynchronize(st), "gather")) return e;
    for (int c = 0; c < ncols; c++) {
        outs[c]->size = (gdf_size_type)n_out;
        outs[c]->null_count = outs[c]->valid ? (gdf_size_type)(n_out - (int64_t)h[c]) : 0;
        if (frame[c]->dtype == GDF_STRING_CATEGORY) outs[c]->dtype_info.category = frame[c]->dtype_info.category;
    }
    return kSuccess;
}

int process_filter_unfused(gdf_column* const* frame, int ncols, const std::string& cond, gdf_column* const* outs,
                           gdf_size_type* n_out_p, cudaStream_t st) {
    const int64_t n = frame[0]->size;
    Stencil s;
    if (int e = make_stencil(frame, ncols, cond, s, st)) return e;
    DeviceBuffer idx;
    int64_t n_out = 0;
    if (int e = compact(s, n, idx, n_out, st)) return e;
    if (int e = gather_all(frame, ncols, (const int32_t*)idx.p, n_out, outs, st)) return e;
    *n_out_p = (gdf_size_type)n_out;
    return kSuccess;
}

// The reference's two steps for LogicalProject over LogicalFilter: the filtered frame is
// materialised in temporaries, then the projection runs over it.  Kept as a cross-check.
int filter_project_unfused(gdf_column* const* frame, int ncols, const std::string& cond, const char* project_q,
                           gdf_column* const* outs, int n_outs, gdf_size_type* n_out, cudaStream_t st) {
    const int64_t n = frame[0]->size;
    std::vector<gdf_column> tmp(ncols);
    std::vector<DeviceBuffer> bufs(2 * ncols);
    std::vector<gdf_column*> tp(ncols);
    for (int c = 0; c < ncols; c++) {
        tmp[c] = *frame[c];
        if (int e = bufs[2 * c].alloc((size_t)n * gdf_dtype_size(frame[c]->dtype), st)) return e;
        tmp[c].data = bufs[2 * c].p;
        if (frame[c]->valid) {
            if (int e = bufs[2 * c + 1].alloc(gdf_valid_allocation_size(n), st)) return e;
            tmp[c].valid = (gdf_valid_type*)bufs[2 * c + 1].p;
        }
        tp[c] = &tmp[c];
    }
    if (int e = process_filter_unfused(frame, ncols, cond, tp.data(), n_out, st)) return e;
    std::vector<gdf_dtype> f(ncols);
    for (int c = 0; c < ncols; c++) f[c] = frame[c]->dtype;
    category_planning(project_q);
    ProjectPlan pp = plan_project(project_q, f);
    std::vector<gdf_column*> evald;
    for (size_t i = 0; i < pp.columns.size(); i++)
        if (pp.columns[i].first) { outs[i]->size = *n_out; evald.push_back(outs[i]); }
    std::vector<int64_t> nulls(evald.size(), 0);
    if (!evald.empty() && *n_out > 0) {
        std::vector<gdf_column*> ins;
        for (int c : pp.input_columns) ins.push_back(tp[c]);
        ProgramArrays pa{pp.pv.left.data(), pp.pv.right.data(), pp.pv.outs.data(), (int32_t)pp.pv.left.size(),
                         pp.pv.final_pos.data(), pp.pv.bops.data(), pp.pv.uops.data(), pp.pv.lscalars.data(),
                         pp.pv.rscalars.data()};
        EvalOptions eo;
        eo.stream = st;
        eo.null_counts = nulls.data();
        if (int e = perform_operation(evald.data(), (int)evald.size(), ins.data(), (int)ins.size(), pa, eo)) return e;
    }
    for (int i = 0, k = 0; i < n_outs; i++) {
        gdf_column* o = outs[i];
        if (pp.columns[i].first) {
            o->size = *n_out;
            o->null_count = (gdf_size_type)nulls[k++];
        } else {
            const gdf_column* src = tp[pp.columns[i].second];
            const size_t bytes = (size_t)(*n_out) * gdf_dtype_size(src->dtype);
            if (bytes) cudaMemcpyAsync(o->data, src->data, bytes, cudaMemcpyDeviceToDevice, st);
            if (src->valid && o->valid)
                cudaMemcpyAsync(o->valid, src->valid, gdf_valid_allocation_size(*n_out), cudaMemcpyDeviceToDevice, st);
            o->size = *n_out;
            o->null_count = src->null_count;
        }
    }
    return check_cuda(cudaStreamSynchronize(st), "filter_project");
}

// Predicate part of a FilterSpec from the condition text.
int predicate_spec(gdf_column* const* frame, int ncols, const std::string& cond, FilterSpec& spec, Program& pred,
                   bool& have_pred) {
    ExpressionPlan ep = plan_expression(cond, ncols);
    have_pred = false;
    if (ep.clone) {
        if (gdf_dtype_size(frame[ep.clone_column]->dtype) != 1)
            return set_error(kUnsupported, "a bare \"$k\" condition needs a one-byte column (the stencil is read as BOOL8)");
        spec.clone_stencil = true;
        spec.clone_column = ep.clone_column;
        return kSuccess;
    }
    // the stencil the reference evaluates into: INT8 with a validity mask
    gdf_column stencil{};
    stencil.dtype = GDF_INT8;
    stencil.valid = (gdf_valid_type*)(uintptr_t)64;  // never dereferenced: only its presence matters here
    stencil.size = frame[0]->size;
    gdf_column* souts[1] = {&stencil};
    std::vector<gdf_column*> ins;
    for (int c : ep.input_columns) ins.push_back(frame[c]);
    ProgramArrays pa{ep.pv.left.data(), ep.pv.right.data(), ep.pv.outs.data(), (int32_t)ep.pv.left.size(),
                     ep.pv.final_pos.data(), ep.pv.bops.data(), ep.pv.uops.data(), ep.pv.lscalars.data(),
                     ep.pv.rscalars.data()};
    if (int e = build_program(pred, souts, 1, ins.data(), (int)ins.size(), pa, false)) return e;
    spec.predicate_cols = ep.input_columns;
    have_pred = true;
    return kSuccess;
}

void frame_spec(gdf_column* const* frame, int ncols, FilterSpec& spec) {
    spec.n_frame = ncols;
    for (int c = 0; c < ncols; c++) {
        spec.frame_dtypes.push_back(frame[c]->dtype);
        spec.frame_has_valid.push_back(frame[c]->valid != nullptr);
    }
}

bool aligned_to(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

// Everything a fused filter call needs that depends only on the query text and the frame's
// shape (dtypes, masks, null counts being zero or not, alignment) and the outputs' shape.
struct PreparedFilter {
    FilterSpec spec;
    Program pred, proj;
    bool have_pred = false, have_proj = false;
    GeneratedKernel gk;
    const CompiledKernel* k = nullptr;
    // the same filter in grid mode (Shape::grid_k), for synchronous calls whose blocks all fit
    // on the device at once: its shape is chosen with the plan, the kernel compiled on the first
    // call that can use it (null where the size class is large or the shape does not allow it)
    Shape grid_shape;
    mutable std::once_flag grid_once;
    mutable GeneratedKernel gk_grid;
    mutable const CompiledKernel* k_grid = nullptr;
};

std::mutex g_prep_mu;
std::unordered_map<std::string, std::unique_ptr<PreparedFilter>> g_prepared;

// Per-thread device scratch for the look-back states, grown on demand and reused: the
// synchronous entry points finish with it before they return.
struct ThreadScratch {
    void* p = nullptr;
    size_t bytes = 0;
    unsigned long long* head = nullptr;  // page-locked: the header copy back is a plain DMA
    size_t head_words = 0;
};
thread_local std::unordered_map<int, ThreadScratch> t_scratch;

// The calling thread's page-locked header buffer on the current device (at least `words`).
int header_get(size_t words, unsigned long long** out) {
    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    ThreadScratch& ts = t_scratch[dev];
    if (ts.head_words < words) {
        if (ts.head) cudaFreeHost(ts.head);
        ts.head = nullptr;
        ts.head_words = 0;
        const size_t want = std::max<size_t>(words, 128);
        if (int e = check_cuda(cudaMallocHost((void**)&ts.head, want * 8), "cudaMallocHost")) return e;
        ts.head_words = want;
    }
    *out = ts.head;
    return kSuccess;
}

int scratch_get(size_t bytes, cudaStream_t st, void** out) {
    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    ThreadScratch& ts = t_scratch[dev];
    if (ts.bytes < bytes) {
        if (ts.p) cudaFreeAsync(ts.p, st);
        ts.p = nullptr;
        ts.bytes = 0;
        const size_t want = std::max<size_t>(bytes + bytes / 4, 1 << 16);
        if (int e = check_cuda(cudaMallocAsync(&ts.p, want, st), "cudaMallocAsync")) return e;
        ts.bytes = want;
    }
    *out = ts.p;
    return kSuccess;
}

std::string frame_signature(gdf_column* const* frame, int ncols, gdf_column* const* outs, int n_outs) {
    std::string k;
    bool al = true;
    for (int c = 0; c < ncols; c++) {
        k += (char)('A' + (int)frame[c]->dtype);
        k += frame[c]->valid ? (frame[c]->null_count ? 'n' : 'v') : '-';
        if (frame[c]->data && !aligned_to(frame[c]->data, 16)) al = false;
    }
    k += al ? "|a|" : "|u|";
    for (int q = 0; q < n_outs; q++) {
        k += (char)('A' + (int)outs[q]->dtype);
        k += outs[q]->valid ? 'v' : '-';
    }
    // string literals resolve to codes of the category columns' dictionaries
    k += category_key(frame, ncols);
    return k;
}

// Slices per warp chunk for n rows: up to the shape's maximum, smaller for small frames so that
// the chunks are about as many as the resident warps (152 SMs x 40): more, smaller chunks only
// lengthen the look-back chains -- 1M rows (C1) ran 75.5 / 66.6 / 59.6 / 63.9 us per call at
// 64 / 128 / 256 / 512-row chunks.
int chunk_slices(int64_t n, int G) {
    const int64_t target = n / (152 * 16);
    int J = 1;
    while (J < 64 / G && (int64_t)32 * G * J * 2 <= target) J *= 2;
    return J;
}

// Launch-shape overrides for tuning sweeps: RAL_FILTER_TUNE="J=16,U=4,T=256,B=2,S=0"
// (J: slices per chunk, U: predicate-pass unroll, T: threads, B: min blocks per SM,
// S: stage dense slices through shared memory).
std::string filter_tune() {
    const char* v = std::getenv("RAL_FILTER_TUNE");
    return v ? std::string(v) : std::string();
}

void apply_tune(Shape& sh, const std::string& t) { apply_shape_tune(sh, t); }

// Launch shape of a fused filter over n rows (n < 0: large), before RAL_FILTER_TUNE.
Shape default_filter_shape(const FilterSpec& spec, bool aligned16, int64_t n) {
    Shape sh;
    sh.G = aligned16 ? 16 / filter_max_width(spec) : 1;
    sh.threads = 256;
    // Pass 2 walks the chunk's kept-row list (Shape::dense) and a warp pipelines two chunks (pass 1
    // of the next before the look-back of the last), which needs chunks of at most 32 mask words:
    // 1024-row chunks, five resident blocks (47 registers with the 12-op projection).  Measured on
    // the 200M-row filter + project, s = 0.01 / 0.5 / 0.99: 0.54 / 1.83 / 3.11 ms, against
    // 0.63 / 1.81 / 3.12 at six blocks (whose 40-register cap spills) and 0.73 / 1.98 / 3.23
    // unpipelined; on the 500M-row six-column gather 1.36 / 3.67 / 5.57 ms against 2.34 / 5.01 /
    // 6.41 with the slice-wise pass 2 at 2048-row chunks and two blocks.
    const int jmax = std::max(1, 32 / sh.G);
    sh.J = n < 0 ? jmax : std::max(1, std::min(jmax, chunk_slices(n, sh.G)));
    sh.min_blocks = 5;
    sh.unroll = spec.project != nullptr ? 2 : 4;
    sh.stage = false;
    return sh;
}

// Size classes up to this many rows also get the grid-mode kernel.  Its pass 1 reads the whole
// table before any pass 2 starts, so the predicate columns should still be in L2 by then.
constexpr int64_t kGridModeMaxRows = (int64_t)1 << 23;

// Finishes a PreparedFilter whose spec (frame, predicate, projection, outputs) is filled in, for
// calls of n_shape rows (the shape) up to n_max rows (the size class).
int prepare_kernel(PreparedFilter& pf, bool aligned16, int64_t n_shape, int64_t n_max) {
    Shape sh = default_filter_shape(pf.spec, aligned16, n_shape);
    apply_tune(sh, filter_tune());
    const int tuned_k = sh.grid_k;
    sh.grid_k = 0;
    pf.gk = generate_filter_kernel(pf.spec, sh);
    std::string err;
    pf.k = jit_get(pf.gk, err);
    if (!pf.k) return set_error(kJitError, err);
    // grid mode: K chunks per warp so that the class's largest call needs at most the blocks that
    // min_blocks per SM give (checked again against the real occupancy at launch); RAL_FILTER_TUNE
    // R=0 turns it off, R=K forces K
    pf.grid_shape = sh;
    if (n_max <= kGridModeMaxRows || tuned_k > 0) {
        const int64_t wt = filter_tile_rows(sh);
        const int64_t warps = (int64_t)device_sms() * std::max(1, sh.min_blocks) * (sh.threads / 32);
        const int64_t chunks = (std::max<int64_t>(n_max, 1) + wt - 1) / wt;
        pf.grid_shape.grid_k = tuned_k > 0 ? tuned_k : (int)std::max<int64_t>(1, (chunks + warps - 1) / warps);
        if (filter_tune().find("R=0") != std::string::npos || pf.grid_shape.grid_k > 16) pf.grid_shape.grid_k = 0;
    }
    return kSuccess;
}

// The grid-mode kernel of a prepared filter, compiled once on first use; null when the shape has
// no grid mode or it failed to compile (the call then takes the look-back kernel).
const CompiledKernel* grid_kernel(const PreparedFilter& pf) {
    std::call_once(pf.grid_once, [&] {
        if (pf.grid_shape.grid_k <= 0) return;
        GeneratedKernel gg = generate_filter_kernel(pf.spec, pf.grid_shape);
        if (gg.shape.grid_k <= 0) return;
        std::string err;
        pf.gk_grid = std::move(gg);
        pf.k_grid = jit_get(pf.gk_grid, err);
    });
    return pf.k_grid;
}

// Per thread and device: the grid-mode scratch (barrier counter, error count, kept count, valid
// counts, one status word per block).  The barrier counter only grows, so the area is zeroed
// once and then only after a failed call; `epoch` is the counter's value before the next launch.
struct GridArea {
    void* p = nullptr;
    size_t words = 0;
    uint64_t epoch = 0;
    uint64_t err_seen = 0;
    bool dirty = true;
    // page-locked, mapped: the kernel's last block writes the header here, then the tag (word 0)
    unsigned long long* hmap = nullptr;
    unsigned long long* dmap = nullptr;
};
thread_local std::unordered_map<int, GridArea> t_grid;
constexpr size_t kGridAreaWords = 3 + 64 + 8192;
std::atomic<int64_t> g_grid_launches{0};

// A synchronous caller's request for grid mode (no other launch may share the calling thread's
// grid area meanwhile): whether it was used, and the area's error count before the launch.
struct GridCall {
    bool used = false;
    uint64_t err_base = 0;
    const unsigned long long* hmap = nullptr;  // the header, complete once hmap[0] == tag
    uint64_t tag = 0;
};

// The grid-mode launch of a prepared filter over n rows, if its blocks fit on the device at once.
int grid_blocks(const PreparedFilter& pf, int64_t n) {
    if (pf.grid_shape.grid_k <= 0 || n <= 0 || !grid_kernel(pf)) return 0;
    const Shape& gs = pf.gk_grid.shape;
    const int64_t per_block = filter_tile_rows(gs) * (gs.threads / 32) * gs.grid_k;
    const int64_t need = (n + per_block - 1) / per_block;
    const int64_t cap = (int64_t)blocks_per_sm(*pf.k_grid, gs.threads) * device_sms();
    if (need > cap || need + 3 + 64 > (int64_t)kGridAreaWords) return 0;
    return (int)need;
}

// Scratch words a prepared filter needs over n rows: the header and one status word per chunk.
int64_t prepared_scratch_words(const PreparedFilter& pf, int64_t n) {
    const int64_t tile_rows = filter_tile_rows(pf.gk.shape);
    return filter_scratch_header((int)pf.spec.outputs.size()) + (n + tile_rows - 1) / tile_rows;
}

// Enqueues a prepared fused filter over the frame on st: zeroes `scratch` (prepared_scratch_words)
// and the output masks, launches with kept row j written at row obase + j of the outputs (obase in
// 0 .. 31: a chunk that continues a mask word earlier rows have started; the data pointers are
// taken obase rows lower, so row j still lands at element j), and copies the header -- kept count,
// error word, valid counts -- to host_header.  ev (optional) brackets the launch.
int enqueue_prepared(const PreparedFilter& pf, gdf_column* const* frame, gdf_column* const* outs, void* scratch,
                     int obase, unsigned long long* host_header, cudaStream_t st, cudaEvent_t* ev,
                     GridCall* grid_call = nullptr) {
    const int64_t n = frame[0]->size;
    const FilterSpec& spec = pf.spec;
    const int NO = (int)spec.outputs.size();
    for (int c = 0; c < spec.n_frame; c++)
        if (frame[c]->valid && !aligned_to(frame[c]->valid, 4))
            return set_error(kInvalidArgument, "validity masks must be 4-byte aligned");
    for (int q = 0; q < NO; q++)
        if (outs[q]->valid && !aligned_to(outs[q]->valid, 4))
            return set_error(kInvalidArgument, "validity masks must be 4-byte aligned");
    if (obase < 0 || obase > 31) return set_error(kInvalidArgument, "output row offset out of range");
    const int gblocks = grid_call ? grid_blocks(pf, n) : 0;
    const GeneratedKernel& gk = gblocks ? pf.gk_grid : pf.gk;
    const ParamLayout& L = gk.layout;
    const int64_t tile_rows = filter_tile_rows(gk.shape);
    const int64_t header = filter_scratch_header(NO);
    GridArea* area = nullptr;
    if (gblocks) {
        // grid mode: the kernel zeroes the output masks and valid counts itself; the area is
        // zeroed only when new or after a failed call
        int dev = 0;
        if (int e = check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return e;
        area = &t_grid[dev];
        if (!area->p) {
            if (int e = check_cuda(cudaMalloc(&area->p, kGridAreaWords * 8), "cudaMalloc")) return e;
            area->words = kGridAreaWords;
            area->dirty = true;
        }
        if (!area->hmap) {
            if (int e = check_cuda(cudaHostAlloc((void**)&area->hmap, 128 * 8, cudaHostAllocMapped), "cudaHostAlloc"))
                return e;
            if (int e = check_cuda(cudaHostGetDevicePointer((void**)&area->dmap, area->hmap, 0),
                                   "cudaHostGetDevicePointer"))
                return e;
        }
        if (area->dirty) {
            if (int e = check_cuda(cudaMemsetAsync(area->p, 0, area->words * 8, st), "cudaMemsetAsync")) return e;
            area->epoch = 0;
            area->err_seen = 0;
            area->dirty = false;
        }
        scratch = area->p;
        grid_call->used = true;
        grid_call->err_base = area->err_seen;
        grid_call->hmap = area->hmap;
        grid_call->tag = area->epoch + 2ull * (uint64_t)gblocks;
        __atomic_store_n(&area->hmap[0], 0ull, __ATOMIC_RELEASE);  // no earlier call's tag can match
    } else {
        if (grid_call) grid_call->used = false;
        cudaMemsetAsync(scratch, 0, (size_t)prepared_scratch_words(pf, n) * 8, st);
        // output masks are assembled with OR at the edges of each warp's range: start from zero
        for (int q = 0; q < NO; q++)
            if (spec.outputs[q].has_valid) cudaMemsetAsync(outs[q]->valid, 0, (size_t)((n + obase + 31) / 32) * 4, st);
    }

    std::vector<uint64_t> slots(L.total, 0);
    slots[L.n_rows] = (uint64_t)n;
    for (int c = 0; c < spec.n_frame; c++) {
        slots[L.in_data + c] = (uint64_t)(uintptr_t)frame[c]->data;
        slots[L.in_valid + c] = (uint64_t)(uintptr_t)frame[c]->valid;
    }
    for (int q = 0; q < NO; q++) {
        const uintptr_t d = (uintptr_t)outs[q]->data - (uintptr_t)obase * gdf_dtype_size(outs[q]->dtype);
        slots[L.out_data + q] = (uint64_t)d;
        slots[L.out_valid + q] = (uint64_t)(uintptr_t)outs[q]->valid;
    }
    slots[L.scratch] = (uint64_t)(uintptr_t)scratch;
    if (L.obase >= 0) slots[L.obase] = (uint64_t)obase;
    if (gblocks) {
        slots[L.epoch] = area->epoch;
        slots[L.hostmap] = (uint64_t)(uintptr_t)area->dmap;
    }
    if (pf.have_pred) fill_scalars(pf.pred, L, slots);
    if (pf.have_proj) {
        ParamLayout QL;
        QL.lscalar_slot = gk.layout_project_lscalar;
        QL.rscalar_slot = gk.layout_project_rscalar;
        QL.rdiv_slot = gk.layout_project_rdiv;
        fill_scalars(pf.proj, QL, slots);
    }
    void* args[] = {slots.data()};
    if (ev) cudaEventRecord(ev[0], st);
    if (gblocks) {
        // every block must be resident for the grid barrier: a cooperative launch guarantees it
        if (int e = check_cuda(cudaLaunchCooperativeKernel((const void*)pf.k_grid->kernel, dim3(gblocks),
                                                           dim3(gk.shape.threads), args, 0, st),
                               "cooperative launch of the filter kernel")) {
            area->dirty = true;
            return e;
        }
        area->epoch += 2ull * (uint64_t)gblocks;  // the barrier step and the completion step
        g_grid_launches++;
    } else {
        const int grid = launch_blocks(*pf.k, gk.shape.threads, tile_rows * (gk.shape.threads / 32), n);
        if (int e = check_cuda(cudaLaunchKernel((const void*)pf.k->kernel, dim3(grid), dim3(gk.shape.threads), args, 0, st),
                               "launch of the filter kernel"))
            return e;
    }
    if (ev) cudaEventRecord(ev[1], st);
    note_launch();
    if (gblocks) return kSuccess;  // the header arrives through the mapped buffer
    return check_cuda(cudaMemcpyAsync(host_header, scratch, (size_t)header * 8, cudaMemcpyDeviceToHost, st),
                      "cudaMemcpyAsync");
}

// Sizes, null counts and dictionaries of a prepared filter's outputs from its header.
void finish_outputs(const PreparedFilter& pf, gdf_column* const* frame, gdf_column* const* outs,
                    const unsigned long long* hp, int64_t n_out) {
    const FilterSpec& spec = pf.spec;
    for (size_t q = 0; q < spec.outputs.size(); q++) {
        outs[q]->size = (gdf_size_type)n_out;
        outs[q]->null_count = spec.outputs[q].has_valid ? (gdf_size_type)(n_out - (int64_t)hp[3 + q]) : 0;
        // a gathered string-category column keeps its source's dictionary (codes unchanged)
        if (!spec.outputs[q].from_project && frame[spec.outputs[q].index]->dtype == GDF_STRING_CATEGORY)
            outs[q]->dtype_info.category = frame[spec.outputs[q].index]->dtype_info.category;
    }
}

// Launches a prepared fused filter over the frame and waits for it.
int run_prepared(const PreparedFilter& pf, gdf_column* const* frame, gdf_column* const* outs, gdf_size_type* n_out_p,
                 cudaStream_t st) {
    const int64_t n = frame[0]->size;
    const int64_t header = filter_scratch_header((int)pf.spec.outputs.size());
    void* scratch = nullptr;
    if (int e = scratch_get((size_t)prepared_scratch_words(pf, n) * 8, st, &scratch)) return e;
    const bool timing = call_timing_enabled();
    call_timing_mark_prepared();
    const auto t_enq0 = std::chrono::steady_clock::now();
    thread_local cudaEvent_t ev[2] = {nullptr, nullptr};
    if (timing && !ev[0]) {
        cudaEventCreate(&ev[0]);
        cudaEventCreate(&ev[1]);
    }
    unsigned long long* hp = nullptr;
    if (int e = header_get((size_t)header, &hp)) return e;
    GridCall gc;
    if (int e = enqueue_prepared(pf, frame, outs, scratch, 0, hp, st, timing ? ev : nullptr, &gc)) return e;
    const auto t_wait0 = std::chrono::steady_clock::now();
    if (gc.used) {
        // the completion tag in the mapped header: polled, with the stream's own status checked
        // every few polls, so an error ends the wait and a finished stream ends it too
        for (unsigned spins = 1;; ++spins) {
            if (__atomic_load_n(&gc.hmap[0], __ATOMIC_ACQUIRE) == gc.tag) break;
            if ((spins & 255u) == 0u) {
                const cudaError_t q = cudaStreamQuery(st);
                if (q == cudaSuccess) break;
                if (q != cudaErrorNotReady) return check_cuda(q, "filter kernel");
            }
        }
    }
    if (int e = check_cuda(cudaStreamSynchronize(st), "filter kernel")) return e;
    if (gc.used) {
        if (__atomic_load_n(&gc.hmap[0], __ATOMIC_ACQUIRE) != gc.tag) {
            int dev = 0;
            cudaGetDevice(&dev);
            t_grid[dev].dirty = true;
            return set_error(kCudaError, "filter kernel finished without its completion tag");
        }
        for (int64_t i = 1; i < header; i++) hp[i] = gc.hmap[i];
        hp[0] = 0;
    }
    if (timing) {
        const auto t_end = std::chrono::steady_clock::now();
        float dev_ms = 0.f;
        cudaEventElapsedTime(&dev_ms, ev[0], ev[1]);
        call_timing_add(std::chrono::duration<double, std::micro>(t_wait0 - t_enq0).count(),
                        std::chrono::duration<double, std::micro>(t_end - t_wait0).count(), dev_ms * 1e3);
    }
    if (gc.used) {
        // the error word of the grid area counts the blocks whose barrier wait gave up
        if (hp[1] != gc.err_base) {
            int dev = 0;
            cudaGetDevice(&dev);
            t_grid[dev].err_seen = hp[1];
            t_grid[dev].dirty = true;
            return set_error(kTimeout, "filter grid barrier wait gave up");
        }
    } else if (hp[1]) {
        return set_error(kTimeout, "filter look-back wait gave up");
    }
    const int64_t n_out = (int64_t)hp[2];
    finish_outputs(pf, frame, outs, hp, n_out);
    *n_out_p = (gdf_size_type)n_out;
    return kSuccess;
}

// Looks up or builds the prepared plan.  `build` fills spec/programs of a fresh plan.
template <typename Build>
int prepared(const std::string& key0, bool aligned16, int64_t n, Build&& build, const PreparedFilter** out) {
    // the chunk size depends on the row count: one plan per size class
    int64_t cls = 1;
    while (cls < n && cls < ((int64_t)1 << 40)) cls <<= 1;
    const std::string key = key0 + "#" + std::to_string(cls) + "#" + filter_tune();
    {
        std::lock_guard<std::mutex> lock(g_prep_mu);
        auto it = g_prepared.find(key);
        if (it != g_prepared.end()) { *out = it->second.get(); return kSuccess; }
    }
    auto pf = std::make_unique<PreparedFilter>();
    if (int e = build(*pf)) return e;
    if (int e = prepare_kernel(*pf, aligned16, cls / 2 + 1, cls)) return e;
    std::lock_guard<std::mutex> lock(g_prep_mu);
    auto res = g_prepared.emplace(key, std::move(pf));
    *out = res.first->second.get();
    return kSuccess;
}

// LogicalProject plans by text and frame dtypes (parsing is the costly part of a small call).
std::mutex g_pp_mu;
std::unordered_map<std::string, std::unique_ptr<ProjectPlan>> g_project_plans;

const ProjectPlan& cached_project_plan(const char* project_q, const std::vector<gdf_dtype>& fd,
                                       const std::string& categories) {
    std::string key(project_q);
    key += '|' + categories + '|';
    for (gdf_dtype t : fd) key += (char)('A' + (int)t);
    {
        std::lock_guard<std::mutex> lock(g_pp_mu);
        auto it = g_project_plans.find(key);
        if (it != g_project_plans.end()) return *it->second;
    }
    auto pp = std::make_unique<ProjectPlan>(plan_project(project_q, fd));
    std::lock_guard<std::mutex> lock(g_pp_mu);
    auto res = g_project_plans.emplace(key, std::move(pp));
    return *res.first->second;
}

// The prepared fused LogicalFilter over this frame (every column gathered into outs).
int prepare_filter(gdf_column* const* frame, int ncols, const std::string& cond, gdf_column* const* outs,
                   const std::string& codes, const PreparedFilter** out) {
    const std::string sig = frame_signature(frame, ncols, outs, ncols);
    const bool al = sig.find("|a|") != std::string::npos;
    return prepared("F|" + cond + "|" + sig + "|" + codes, al, frame[0]->size, [&](PreparedFilter& p) {
        frame_spec(frame, ncols, p.spec);
        if (int e = predicate_spec(frame, ncols, cond, p.spec, p.pred, p.have_pred)) return e;
        if (p.have_pred) p.spec.predicate = &p.pred;
        for (int c = 0; c < ncols; c++) {
            FilterOutput o;
            o.from_project = false;
            o.index = c;
            o.dtype = frame[c]->dtype;
            o.has_valid = frame[c]->valid != nullptr;
            p.spec.outputs.push_back(o);
        }
        return (int)kSuccess;
    }, out);
}

int process_filter_fused(gdf_column* const* frame, int ncols, const std::string& cond, gdf_column* const* outs,
                         gdf_size_type* n_out, cudaStream_t st, const std::string& codes) {
    const PreparedFilter* pf = nullptr;
    if (int rc = prepare_filter(frame, ncols, cond, outs, codes, &pf)) return rc;
    return run_prepared(*pf, frame, outs, n_out, st);
}

}  // namespace

int debug_filter_source(gdf_column* const* frame, int ncols, const char* filter_q, const char* project_q,
                        bool compile, std::string& source, std::string& log) {
    const std::string cond = named_expression(filter_q, "condition");
    if (cond.empty()) return set_error(kParseError, "no condition=[...] in the LogicalFilter");
    FilterSpec spec;
    frame_spec(frame, ncols, spec);
    Program pred, proj;
    bool have_pred = false;
    if (int e = predicate_spec(frame, ncols, cond, spec, pred, have_pred)) return e;
    if (have_pred) spec.predicate = &pred;
    std::vector<gdf_column> outcols;
    if (project_q && *project_q) {
        std::vector<gdf_dtype> fd(ncols);
        for (int c = 0; c < ncols; c++) fd[c] = frame[c]->dtype;
        ProjectPlan pp = plan_project(project_q, fd);
        outcols.resize(pp.columns.size());
        std::vector<gdf_column*> evald;
        for (size_t i = 0; i < pp.columns.size(); i++) {
            outcols[i] = gdf_column{};
            const bool ev = pp.columns[i].first;
            outcols[i].dtype = ev ? pp.eval_dtypes[pp.columns[i].second] : fd[pp.columns[i].second];
            outcols[i].valid = (ev || frame[pp.columns[i].second]->valid) ? (gdf_valid_type*)(uintptr_t)64 : nullptr;
            if (ev) evald.push_back(&outcols[i]);
            FilterOutput o;
            o.from_project = ev;
            o.index = pp.columns[i].second;
            o.dtype = outcols[i].dtype;
            o.has_valid = outcols[i].valid != nullptr;
            spec.outputs.push_back(o);
        }
        if (!evald.empty()) {
            std::vector<gdf_column*> ins;
            for (int c : pp.input_columns) ins.push_back(frame[c]);
            ProgramArrays pa{pp.pv.left.data(), pp.pv.right.data(), pp.pv.outs.data(), (int32_t)pp.pv.left.size(),
                             pp.pv.final_pos.data(), pp.pv.bops.data(), pp.pv.uops.data(), pp.pv.lscalars.data(),
                             pp.pv.rscalars.data()};
            if (int e = build_program(proj, evald.data(), (int)evald.size(), ins.data(), (int)ins.size(), pa, true)) return e;
            spec.project = &proj;
            spec.project_cols = pp.input_columns;
        }
    } else {
        for (int c = 0; c < ncols; c++) {
            FilterOutput o;
            o.index = c;
            o.dtype = frame[c]->dtype;
            o.has_valid = frame[c]->valid != nullptr;
            spec.outputs.push_back(o);
        }
    }
    Shape sh = default_filter_shape(spec, true, -1);
    apply_tune(sh, filter_tune());
    GeneratedKernel gk = generate_filter_kernel(spec, sh);
    source = std::string(jit_prelude()) + "\n" + gk.source;
    if (compile) {
        std::string err;
        size_t bytes = 0;
        if (!jit_compile_only(gk, &bytes, &log, err)) {
            log = err;
            return set_error(kJitError, err);
        }
    }
    return kSuccess;
}

int process_filter(gdf_column* const* frame, int ncols, const char* query_part, gdf_column* const* outs,
                   gdf_size_type* n_out, const FilterOptions& opt) {
    call_timing_start();
    if (!frame || ncols <= 0 || !query_part || !outs || !n_out) return set_error(kInvalidArgument, "null argument");
    if (int e = check_outputs(frame, ncols, outs)) return e;
    const std::string cond = named_expression(query_part, "condition");
    if (cond.empty()) return set_error(kParseError, "no condition=[...] in the LogicalFilter");
    CategoryScope categories(frame, ncols);
    // string literals first, once, in the reference's order: a missing one rewrites its column's
    // codes and dictionary; the plans below replay the codes, which the plan caches key on
    categories.planning(cond);
    if (has_string_literal(cond.c_str()) || frame_has_category(frame, ncols)) plan_expression(cond, ncols);
    categories.replay();
    if (frame[0]->size == 0) {
        // the reference leaves an empty frame untouched
        for (int c = 0; c < ncols; c++) { outs[c]->size = 0; outs[c]->null_count = 0; }
        *n_out = 0;
        return kSuccess;
    }
    if (filter_mode(opt) == 1) return process_filter_unfused(frame, ncols, cond, outs, n_out, opt.stream);
    return process_filter_fused(frame, ncols, cond, outs, n_out, opt.stream, categories.recorded_key());
}

int plan_filter_project(gdf_column* const* frame, int ncols, const char* filter_q, const char* project_q,
                        std::unique_ptr<FilterPlan>& plan) {
    if (!frame || ncols <= 0 || !filter_q || !project_q) return set_error(kInvalidArgument, "null argument");
    for (int c = 0; c < ncols; c++) {
        if (!frame[c]) return set_error(kInvalidArgument, "null frame column");
        if (frame[c]->size != frame[0]->size) return set_error(kInvalidArgument, "frame columns differ in size");
        if (gdf_dtype_size(frame[c]->dtype) == 0) return set_error(kUnsupported, "column dtype has no fixed width");
    }
    const std::string cond = named_expression(filter_q, "condition");
    if (cond.empty()) return set_error(kParseError, "no condition=[...] in the LogicalFilter");
    std::vector<gdf_dtype> fd(ncols);
    for (int c = 0; c < ncols; c++) fd[c] = frame[c]->dtype;
    CategoryScope categories(frame, ncols);
    categories.planning(cond);
    if (has_string_literal(cond.c_str()) || frame_has_category(frame, ncols)) plan_expression(cond, ncols);
    categories.planning(project_q);
    if (has_string_literal(project_q) || frame_has_category(frame, ncols)) plan_project(project_q, fd);
    categories.replay();
    const ProjectPlan& pp = cached_project_plan(project_q, fd, category_key(frame, ncols) + categories.recorded_key());
    categories.planning(cond);
    auto p = std::make_unique<FilterPlan>();
    frame_spec(frame, ncols, p->spec);
    if (int e = predicate_spec(frame, ncols, cond, p->spec, p->pred, p->have_pred)) return e;
    if (p->have_pred) p->spec.predicate = &p->pred;
    const int n_outs = (int)pp.columns.size();
    // stand-in output descriptors: only dtype and mask presence matter to the program
    std::vector<gdf_column> stand(n_outs);
    for (int i = 0; i < n_outs; i++) {
        const bool ev = pp.columns[i].first;
        stand[i].dtype = ev ? pp.eval_dtypes[pp.columns[i].second] : fd[pp.columns[i].second];
        const bool mask = ev ? true : frame[pp.columns[i].second]->valid != nullptr;
        stand[i].valid = mask ? (gdf_valid_type*)(uintptr_t)64 : nullptr;
        stand[i].size = frame[0]->size;
        p->out_dtypes.push_back(stand[i].dtype);
        p->out_valid.push_back(mask);
    }
    p->have_proj = !pp.eval_dtypes.empty();
    if (p->have_proj) {
        std::vector<gdf_column*> evald;
        for (int i = 0; i < n_outs; i++)
            if (pp.columns[i].first) evald.push_back(&stand[i]);
        std::vector<gdf_column*> ins;
        for (int c : pp.input_columns) ins.push_back(frame[c]);
        ProgramArrays pa{pp.pv.left.data(), pp.pv.right.data(), pp.pv.outs.data(), (int32_t)pp.pv.left.size(),
                         pp.pv.final_pos.data(), pp.pv.bops.data(), pp.pv.uops.data(), pp.pv.lscalars.data(),
                         pp.pv.rscalars.data()};
        // as in filter_project: the filtered frame's masks are read whenever present
        if (int e = build_program(p->proj, evald.data(), (int)evald.size(), ins.data(), (int)ins.size(), pa, true))
            return e;
        p->spec.project = &p->proj;
        p->spec.project_cols = pp.input_columns;
    }
    for (int i = 0; i < n_outs; i++) {
        FilterOutput o;
        o.from_project = pp.columns[i].first;
        o.index = pp.columns[i].second;
        o.dtype = p->out_dtypes[i];
        o.has_valid = p->out_valid[i];
        p->spec.outputs.push_back(o);
    }
    plan = std::move(p);
    return kSuccess;
}

void filter_fill_slots(const FilterPlan& plan, const GeneratedKernel& gk, gdf_column* const* frame, int64_t n_rows,
                       void* const* out_data, void* const* out_valid, void* scratch, std::vector<uint64_t>& slots) {
    const ParamLayout& L = gk.layout;
    const FilterSpec& spec = plan.spec;
    slots.assign(L.total, 0);
    slots[L.n_rows] = (uint64_t)n_rows;
    for (int c = 0; c < spec.n_frame; c++) {
        slots[L.in_data + c] = (uint64_t)(uintptr_t)frame[c]->data;
        slots[L.in_valid + c] = (uint64_t)(uintptr_t)frame[c]->valid;
    }
    for (size_t q = 0; q < spec.outputs.size(); q++) {
        slots[L.out_data + q] = (uint64_t)(uintptr_t)out_data[q];
        slots[L.out_valid + q] = (uint64_t)(uintptr_t)out_valid[q];
    }
    slots[L.scratch] = (uint64_t)(uintptr_t)scratch;
    if (plan.have_pred) fill_scalars(plan.pred, L, slots);
    if (plan.have_proj) {
        ParamLayout QL;
        QL.lscalar_slot = gk.layout_project_lscalar;
        QL.rscalar_slot = gk.layout_project_rscalar;
        QL.rdiv_slot = gk.layout_project_rdiv;
        fill_scalars(plan.proj, QL, slots);
    }
}

int prepare_filter_project(gdf_column* const* frame, int ncols, const std::string& cond, const char* project_q,
                           const ProjectPlan& pp, gdf_column* const* outs, int n_outs, const std::string& codes,
                           const PreparedFilter** out);

int prepare_filter_project(gdf_column* const* frame, int ncols, const std::string& cond, const char* project_q,
                           const ProjectPlan& pp, gdf_column* const* outs, int n_outs, const std::string& codes,
                           const PreparedFilter** out);

// String literals of a filter + project, resolved once in the reference's order (the filter's
// before the projection's, as process_filter runs before execute_project_plan), then replayed;
// returns the projection's plan, keyed on the recorded codes.
const ProjectPlan& resolve_filter_project(gdf_column* const* frame, int ncols, const std::string& cond,
                                          const char* project_q, const std::vector<gdf_dtype>& fd,
                                          CategoryScope& categories, std::string& codes) {
    const bool cat = frame_has_category(frame, ncols);
    categories.planning(cond);
    if (has_string_literal(cond.c_str()) || cat) plan_expression(cond, ncols);
    categories.planning(project_q);
    if (has_string_literal(project_q) || cat) plan_project(project_q, fd);
    categories.replay();
    codes = categories.recorded_key();
    const ProjectPlan& pp = cached_project_plan(project_q, fd, category_key(frame, ncols) + codes);
    categories.planning(cond);
    return pp;
}

int prepare_standalone_filter(gdf_column* const* frame, int ncols, const char* filter_q, const char* project_q,
                              gdf_column* const* outs, int n_outs, const void** handle) {
    if (!frame || ncols <= 0 || !filter_q || !project_q || !outs || !handle)
        return set_error(kInvalidArgument, "null argument");
    try {
        const std::string cond = named_expression(filter_q, "condition");
        if (cond.empty()) return set_error(kParseError, "no condition=[...] in the LogicalFilter");
        std::vector<gdf_dtype> fd(ncols);
        for (int c = 0; c < ncols; c++) fd[c] = frame[c]->dtype;
        CategoryScope categories(frame, ncols);
        std::string codes;
        const ProjectPlan& pp = resolve_filter_project(frame, ncols, cond, project_q, fd, categories, codes);
        if ((int)pp.columns.size() != n_outs)
            return set_error(kInvalidArgument, "out_columns count differs from the projection's");
        const PreparedFilter* pf = nullptr;
        if (int rc = prepare_filter_project(frame, ncols, cond, project_q, pp, outs, n_outs, codes, &pf)) return rc;
        *handle = pf;
        return kSuccess;
    } catch (const ParseError& e) {
        return set_error(kParseError, e.what());
    }
}

int64_t standalone_scratch_words(const void* handle, int64_t n) {
    return prepared_scratch_words(*static_cast<const PreparedFilter*>(handle), n);
}

int enqueue_standalone_filter(const void* handle, gdf_column* const* frame, gdf_column* const* outs, void* scratch,
                              unsigned long long* host_header, cudaStream_t st) {
    return enqueue_prepared(*static_cast<const PreparedFilter*>(handle), frame, outs, scratch, 0, host_header, st,
                            nullptr);
}

int filter_project(gdf_column* const* frame, int ncols, const char* filter_q, const char* project_q,
                   gdf_column* const* outs, int n_outs, gdf_size_type* n_out, const FilterOptions& opt) {
    call_timing_start();
    if (!frame || ncols <= 0 || !filter_q || !project_q || !outs || !n_out)
        return set_error(kInvalidArgument, "null argument");
    for (int c = 0; c < ncols; c++) {
        if (!frame[c]) return set_error(kInvalidArgument, "null frame column");
        if (frame[c]->size != frame[0]->size) return set_error(kInvalidArgument, "frame columns differ in size");
        if (gdf_dtype_size(frame[c]->dtype) == 0) return set_error(kUnsupported, "column dtype has no fixed width");
    }
    const std::string cond = named_expression(filter_q, "condition");
    if (cond.empty()) return set_error(kParseError, "no condition=[...] in the LogicalFilter");
    std::vector<gdf_dtype> fd(ncols);
    for (int c = 0; c < ncols; c++) fd[c] = frame[c]->dtype;
    CategoryScope categories(frame, ncols);
    std::string codes;
    const ProjectPlan& pp = resolve_filter_project(frame, ncols, cond, project_q, fd, categories, codes);
    if ((int)pp.columns.size() != n_outs) return set_error(kInvalidArgument, "out_columns count differs from the projection's");
    for (int i = 0; i < n_outs; i++) {
        if (!outs[i]) return set_error(kInvalidArgument, "null out column");
        const bool ev = pp.columns[i].first;
        const gdf_dtype want = ev ? pp.eval_dtypes[pp.columns[i].second] : fd[pp.columns[i].second];
        if (outs[i]->dtype != want) return set_error(kInvalidArgument, "out column " + std::to_string(i) + " has the wrong dtype");
        if (!ev && (outs[i]->valid != nullptr) != (frame[pp.columns[i].second]->valid != nullptr))
            return set_error(kInvalidArgument, "a pass-through out column carries a mask exactly when its frame column does");
        if (frame[0]->size > 0 && !outs[i]->data) return set_error(kInvalidArgument, "out column without data");
    }
    if (frame[0]->size == 0) {
        for (int i = 0; i < n_outs; i++) { outs[i]->size = 0; outs[i]->null_count = 0; }
        *n_out = 0;
        return kSuccess;
    }
    if (filter_mode(opt) == 1) return filter_project_unfused(frame, ncols, cond, project_q, outs, n_outs, n_out, opt.stream);
    const PreparedFilter* pf = nullptr;
    if (int rc = prepare_filter_project(frame, ncols, cond, project_q, pp, outs, n_outs, codes, &pf)) return rc;
    return run_prepared(*pf, frame, outs, n_out, opt.stream);
}

// The prepared fused LogicalFilter + LogicalProject over this frame and these outputs.
int prepare_filter_project(gdf_column* const* frame, int ncols, const std::string& cond, const char* project_q,
                           const ProjectPlan& pp, gdf_column* const* outs, int n_outs, const std::string& codes,
                           const PreparedFilter** out) {
    const std::string sig = frame_signature(frame, ncols, outs, n_outs);
    const bool al = sig.find("|a|") != std::string::npos;
    return prepared("FP|" + cond + "|" + std::string(project_q) + "|" + sig + "|" + codes, al, frame[0]->size,
                      [&](PreparedFilter& p) {
        frame_spec(frame, ncols, p.spec);
        if (int e = predicate_spec(frame, ncols, cond, p.spec, p.pred, p.have_pred)) return e;
        if (p.have_pred) p.spec.predicate = &p.pred;
        p.have_proj = !pp.eval_dtypes.empty();
        if (p.have_proj) {
            std::vector<gdf_column*> evald;
            for (int i = 0; i < n_outs; i++)
                if (pp.columns[i].first) evald.push_back(outs[i]);
            std::vector<gdf_column*> ins;
            for (int c : pp.input_columns) ins.push_back(frame[c]);
            ProgramArrays pa{pp.pv.left.data(), pp.pv.right.data(), pp.pv.outs.data(), (int32_t)pp.pv.left.size(),
                             pp.pv.final_pos.data(), pp.pv.bops.data(), pp.pv.uops.data(), pp.pv.lscalars.data(),
                             pp.pv.rscalars.data()};
            // the reference projects the filtered frame, whose null counts are recounted from the
            // gathered masks: a mask is read whenever present
            if (int e = build_program(p.proj, evald.data(), (int)evald.size(), ins.data(), (int)ins.size(), pa, true))
                return e;
            p.spec.project = &p.proj;
            p.spec.project_cols = pp.input_columns;
        }
        for (int i = 0; i < n_outs; i++) {
            FilterOutput o;
            o.from_project = pp.columns[i].first;
            o.index = pp.columns[i].second;
            o.dtype = outs[i]->dtype;
            o.has_valid = outs[i]->valid != nullptr;
            p.spec.outputs.push_back(o);
        }
        return (int)kSuccess;
    }, out);
}


// ---- LogicalFilter (and LogicalProject over it) over columns in host memory ----------------------
//
// The rows stream through the GPU in chunks on three streams, each with its own device area: a
// chunk's copies in, the fused filter kernel over the chunk, then its kept rows copied back to the
// output's running row offset.  That offset is known once the earlier chunks' kept counts are read
// back, so the host reads each chunk's count after its kernel (the copies of the next chunks are
// already under way) and launches the kernel of chunk i with its output rows starting at bit
// (offset mod 32) of the chunk's mask buffer: whole mask words then copy back to their place, and
// the one word a chunk shares with the rows before it is merged on the host at the end.

namespace {

struct HostFilterArea {
    size_t bytes = 0;
    void* dev = nullptr;
    unsigned long long* pinned = nullptr;  // headers of the three slots, then first mask words
    size_t pinned_words = 0;
    cudaStream_t s[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t kernel_done[3] = {nullptr, nullptr, nullptr};
    ~HostFilterArea() {
        if (dev) cudaFree(dev);
        if (pinned) cudaFreeHost(pinned);
        for (int k = 0; k < 3; k++) {
            if (s[k]) cudaStreamDestroy(s[k]);
            if (kernel_done[k]) cudaEventDestroy(kernel_done[k]);
        }
    }
};

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

int64_t filter_grid_launches() { return g_grid_launches.load(); }

int filter_host(gdf_column* const* frame, int ncols, const char* filter_q, const char* project_q,
                gdf_column* const* outs, int n_outs, gdf_size_type* n_out_p, int64_t chunk_rows) {
    if (!frame || ncols <= 0 || !filter_q || !outs || !n_out_p) return set_error(kInvalidArgument, "null argument");
    for (int c = 0; c < ncols; c++) {
        if (!frame[c]) return set_error(kInvalidArgument, "null frame column");
        if (frame[c]->size != frame[0]->size) return set_error(kInvalidArgument, "frame columns differ in size");
        if (gdf_dtype_size(frame[c]->dtype) == 0) return set_error(kUnsupported, "column dtype has no fixed width");
    }
    const std::string cond = named_expression(filter_q, "condition");
    if (cond.empty()) return set_error(kParseError, "no condition=[...] in the LogicalFilter");
    const int64_t n = frame[0]->size;
    std::vector<gdf_dtype> fd(ncols);
    for (int c = 0; c < ncols; c++) fd[c] = frame[c]->dtype;
    // string literals resolve against the host columns' dictionaries; a literal the dictionary lacks
    // (or two category columns with different dictionaries) would rewrite codes, which needs the
    // column on the device: rejected here
    CategoryScope categories(frame, ncols);
    categories.read_only = true;
    categories.planning(cond);
    plan_expression(cond, ncols);
    if (project_q) {
        categories.planning(project_q);
        plan_project(project_q, fd);
    }
    categories.replay();
    const std::string codes = categories.recorded_key();
    // output dtypes and mask presence
    std::vector<gdf_dtype> odt;
    std::vector<bool> ovalid;
    const ProjectPlan* pp = nullptr;
    if (project_q) {
        pp = &cached_project_plan(project_q, fd, category_key(frame, ncols) + codes);
        for (const auto& col : pp->columns) {
            odt.push_back(col.first ? pp->eval_dtypes[col.second] : fd[col.second]);
            ovalid.push_back(col.first ? true : frame[col.second]->valid != nullptr);
        }
    } else {
        for (int c = 0; c < ncols; c++) {
            odt.push_back(fd[c]);
            ovalid.push_back(frame[c]->valid != nullptr);
        }
    }
    const int NO = (int)odt.size();
    if (n_outs != NO) return set_error(kInvalidArgument, "out_columns count differs from the plan's");
    for (int q = 0; q < NO; q++) {
        if (!outs[q]) return set_error(kInvalidArgument, "null out column");
        if (outs[q]->dtype != odt[q]) return set_error(kInvalidArgument, "out column " + std::to_string(q) + " has the wrong dtype");
        if ((outs[q]->valid != nullptr) != ovalid[q])
            return set_error(kInvalidArgument, "out column " + std::to_string(q) + ": a validity buffer is expected exactly "
                                               "when the output has one");
        if (n > 0 && !outs[q]->data) return set_error(kInvalidArgument, "out column without data");
        if (outs[q]->valid && !aligned_to(outs[q]->valid, 4)) return set_error(kInvalidArgument, "masks must be 4-byte aligned");
    }
    for (int c = 0; c < ncols; c++)
        if (n > 0 && !frame[c]->data) return set_error(kInvalidArgument, "frame column without data");
    if (n == 0) {
        for (int q = 0; q < NO; q++) { outs[q]->size = 0; outs[q]->null_count = 0; }
        *n_out_p = 0;
        return kSuccess;
    }
    int64_t C = chunk_rows > 0 ? chunk_rows : ((int64_t)4 << 20);
    C = std::max<int64_t>(1024, (C + 1023) / 1024 * 1024);
    if (C > n) C = (n + 1023) / 1024 * 1024;
    const int64_t nch = (n + C - 1) / C;

    // one device area per stream: the frame's chunk, the outputs' chunk (32 rows of room for the
    // row offset), the filter's scratch
    std::vector<size_t> in_data_off(ncols), in_mask_off(ncols), out_data_off(NO), out_mask_off(NO);
    size_t per_slot = 0;
    for (int c = 0; c < ncols; c++) {
        in_data_off[c] = per_slot;
        per_slot += round256((size_t)C * gdf_dtype_size(fd[c]));
        in_mask_off[c] = per_slot;
        if (frame[c]->valid) per_slot += round256((size_t)gdf_valid_allocation_size(C));
    }
    for (int q = 0; q < NO; q++) {
        out_data_off[q] = per_slot;
        per_slot += round256((size_t)(C + 32) * gdf_dtype_size(odt[q]));
        out_mask_off[q] = per_slot;
        if (ovalid[q]) per_slot += round256((size_t)gdf_valid_allocation_size(C + 64));
    }
    const size_t scratch_off = per_slot;
    // scratch: header + chunk states of the largest plan (the chunk size class bounds the tiles)
    per_slot += round256((size_t)(filter_scratch_header(NO) + C / 32 + 64) * 8);

    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    static thread_local std::map<int, HostFilterArea> areas;
    HostFilterArea& A = areas[dev];
    for (int k = 0; k < 3; k++) {
        if (!A.s[k] && check_cuda(cudaStreamCreateWithFlags(&A.s[k], cudaStreamNonBlocking), "cudaStreamCreate"))
            return kCudaError;
        if (!A.kernel_done[k] &&
            check_cuda(cudaEventCreateWithFlags(&A.kernel_done[k], cudaEventDisableTiming), "cudaEventCreate"))
            return kCudaError;
    }
    if (A.bytes < 3 * per_slot) {
        if (A.dev) cudaFree(A.dev);
        A.dev = nullptr;
        A.bytes = 0;
        if (int e = check_cuda(cudaMalloc(&A.dev, 3 * per_slot), "cudaMalloc")) return e;
        A.bytes = 3 * per_slot;
    }
    const int64_t header = filter_scratch_header(NO);
    const size_t want_pinned = (size_t)(3 * header + nch * NO + 8);
    if (A.pinned_words < want_pinned) {
        if (A.pinned) cudaFreeHost(A.pinned);
        A.pinned = nullptr;
        A.pinned_words = 0;
        if (int e = check_cuda(cudaMallocHost((void**)&A.pinned, want_pinned * 8), "cudaMallocHost")) return e;
        A.pinned_words = want_pinned;
    }
    auto slot_base = [&](int k) { return (char*)A.dev + (size_t)k * per_slot; };
    uint32_t* first_words = (uint32_t*)(A.pinned + 3 * header);  // nch x NO words

    // per slot: the device descriptors of the chunk frame and outputs
    std::vector<gdf_column> dframe(3 * ncols), douts(3 * NO);
    std::vector<gdf_column*> pframe(3 * ncols), pouts(3 * NO);
    for (int k = 0; k < 3; k++) {
        for (int c = 0; c < ncols; c++) {
            gdf_column& d = dframe[k * ncols + c];
            d = *frame[c];  // dtype, null_count (read by the validity pass), dictionary
            d.data = slot_base(k) + in_data_off[c];
            d.valid = frame[c]->valid ? (gdf_valid_type*)(slot_base(k) + in_mask_off[c]) : nullptr;
            pframe[k * ncols + c] = &d;
        }
        for (int q = 0; q < NO; q++) {
            gdf_column& d = douts[k * NO + q];
            d = *outs[q];
            d.data = slot_base(k) + out_data_off[q];
            d.valid = ovalid[q] ? (gdf_valid_type*)(slot_base(k) + out_mask_off[q]) : nullptr;
            pouts[k * NO + q] = &d;
        }
    }
    auto rows_of = [&](int64_t i) { return std::min<int64_t>(C, n - i * C); };
    auto copy_in = [&](int64_t i) -> int {
        const int k = (int)(i % 3);
        const int64_t r0 = i * C, rows = rows_of(i);
        for (int c = 0; c < ncols; c++) {
            const int w = gdf_dtype_size(fd[c]);
            if (int e = check_cuda(cudaMemcpyAsync(slot_base(k) + in_data_off[c], (const char*)frame[c]->data + r0 * w,
                                                   (size_t)(rows * w), cudaMemcpyHostToDevice, A.s[k]),
                                   "cudaMemcpyAsync"))
                return e;
            if (frame[c]->valid)
                if (int e = check_cuda(cudaMemcpyAsync(slot_base(k) + in_mask_off[c], (const char*)frame[c]->valid + r0 / 8,
                                                       (size_t)((rows + 7) / 8), cudaMemcpyHostToDevice, A.s[k]),
                                       "cudaMemcpyAsync"))
                    return e;
        }
        return kSuccess;
    };
    for (int64_t i = 0; i < std::min<int64_t>(3, nch); i++)
        if (int e = copy_in(i)) return e;

    struct ChunkOut {
        int64_t offset, kept, words;
    };
    std::vector<ChunkOut> done;
    done.reserve(nch);
    std::vector<int64_t> valid_count(NO, 0);
    int64_t offset = 0;
    for (int64_t i = 0; i < nch; i++) {
        const int k = (int)(i % 3);
        const int64_t rows = rows_of(i);
        for (int c = 0; c < ncols; c++) dframe[k * ncols + c].size = (gdf_size_type)rows;
        const PreparedFilter* pf = nullptr;
        int rc = project_q ? prepare_filter_project(&pframe[k * ncols], ncols, cond, project_q, *pp, &pouts[k * NO], NO,
                                                    codes, &pf)
                           : prepare_filter(&pframe[k * ncols], ncols, cond, &pouts[k * NO], codes, &pf);
        if (rc) return rc;
        if ((int64_t)prepared_scratch_words(*pf, rows) * 8 > (int64_t)(per_slot - scratch_off))
            return set_error(kInvalidArgument, "filter scratch larger than its area");
        const int obase = (int)(offset & 31);
        unsigned long long* hdr = A.pinned + k * header;
        if (int e = enqueue_prepared(*pf, &pframe[k * ncols], &pouts[k * NO], slot_base(k) + scratch_off, obase, hdr,
                                     A.s[k], nullptr))
            return e;
        if (int e = check_cuda(cudaEventRecord(A.kernel_done[k], A.s[k]), "cudaEventRecord")) return e;
        if (int e = check_cuda(cudaEventSynchronize(A.kernel_done[k]), "filter kernel")) return e;
        if (hdr[1]) return set_error(kTimeout, "filter look-back wait gave up");
        const int64_t kept = (int64_t)hdr[2];
        const int64_t words = (obase + kept + 31) / 32;
        for (int q = 0; q < NO; q++) {
            valid_count[q] += ovalid[q] ? (int64_t)hdr[3 + q] : 0;
            const int w = gdf_dtype_size(odt[q]);
            if (kept > 0)
                if (int e = check_cuda(cudaMemcpyAsync((char*)outs[q]->data + offset * w, slot_base(k) + out_data_off[q],
                                                       (size_t)(kept * w), cudaMemcpyDeviceToHost, A.s[k]),
                                       "cudaMemcpyAsync"))
                    return e;
            if (!ovalid[q]) continue;
            // word 0 (shared with the rows before the chunk) to the pinned area, words 1.. to their place
            const char* dm = slot_base(k) + out_mask_off[q];
            if (int e = check_cuda(cudaMemcpyAsync(first_words + i * NO + q, dm, 4, cudaMemcpyDeviceToHost, A.s[k]),
                                   "cudaMemcpyAsync"))
                return e;
            if (words > 1)
                if (int e = check_cuda(cudaMemcpyAsync((uint32_t*)outs[q]->valid + offset / 32 + 1, dm + 4,
                                                       (size_t)(words - 1) * 4, cudaMemcpyDeviceToHost, A.s[k]),
                                       "cudaMemcpyAsync"))
                    return e;
        }
        done.push_back({offset, kept, words});
        offset += kept;
        // the stream's next chunk goes in after this chunk's copies back (stream order)
        if (i + 3 < nch)
            if (int e = copy_in(i + 3)) return e;
    }
    for (int k = 0; k < 3; k++)
        if (int e = check_cuda(cudaStreamSynchronize(A.s[k]), "cudaStreamSynchronize")) return e;
    // merge each chunk's first mask word into the output: a word no copy has written yet starts at 0
    for (int q = 0; q < NO; q++) {
        if (!ovalid[q]) continue;
        uint32_t* hv = (uint32_t*)outs[q]->valid;
        int64_t last_written = -1, last_zeroed = -1;
        for (int64_t i = 0; i < nch; i++) {
            const int64_t W = done[i].offset / 32;
            if (W > last_written && W != last_zeroed) {
                hv[W] = 0;
                last_zeroed = W;
            }
            hv[W] |= first_words[i * NO + q];
            if (done[i].words > 1) last_written = W + done[i].words - 1;
        }
    }
    for (int q = 0; q < NO; q++) {
        outs[q]->size = (gdf_size_type)offset;
        outs[q]->null_count = ovalid[q] ? (gdf_size_type)(offset - valid_count[q]) : 0;
        if (!(project_q && pp->columns[q].first)) {
            const int src = project_q ? pp->columns[q].second : q;
            if (frame[src]->dtype == GDF_STRING_CATEGORY) outs[q]->dtype_info.category = frame[src]->dtype_info.category;
        }
    }
    *n_out_p = (gdf_size_type)offset;
    return kSuccess;
}

}  // namespace ral
