// filter.cpp — LogicalFilter: stencil, compaction and gather of every column.
//
// Reference flow (src/CalciteInterpreter.cpp:509-573): evaluate the condition
// into an INT8 stencil with a validity mask, build an int32 iota, compact it
// with cudf::apply_boolean_mask (row kept when the stencil bit is valid and
// the byte is nonzero), then materialize_column every frame column.
#include "filter.h"

#include <cstdlib>
#include <string>
#include <vector>

#include "engine.h"
#include "frontend.h"
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

}  // namespace

int process_filter_fused(gdf_column* const* frame, int ncols, const std::string& cond, gdf_column* const* outs,
                         gdf_size_type* n_out, cudaStream_t st);

int process_filter(gdf_column* const* frame, int ncols, const char* query_part, gdf_column* const* outs,
                   gdf_size_type* n_out, const FilterOptions& opt) {
    if (!frame || ncols <= 0 || !query_part || !outs || !n_out) return set_error(kInvalidArgument, "null argument");
    if (int e = check_outputs(frame, ncols, outs)) return e;
    const std::string cond = named_expression(query_part, "condition");
    if (cond.empty()) return set_error(kParseError, "no condition=[...] in the LogicalFilter");
    if (frame[0]->size == 0) {
        // the reference leaves an empty frame untouched
        for (int c = 0; c < ncols; c++) { outs[c]->size = 0; outs[c]->null_count = 0; }
        *n_out = 0;
        return kSuccess;
    }
    if (filter_mode(opt) == 1) return process_filter_unfused(frame, ncols, cond, outs, n_out, opt.stream);
    return process_filter_fused(frame, ncols, cond, outs, n_out, opt.stream);
}

int process_filter_fused(gdf_column* const* frame, int ncols, const std::string& cond, gdf_column* const* outs,
                         gdf_size_type* n_out, cudaStream_t st) {
    // fused kernel not built yet: the three-step path
    return process_filter_unfused(frame, ncols, cond, outs, n_out, st);
}

int filter_project(gdf_column* const* frame, int ncols, const char* filter_q, const char* project_q,
                   gdf_column* const* outs, int n_outs, gdf_size_type* n_out, const FilterOptions& opt) {
    if (!frame || ncols <= 0 || !filter_q || !project_q || !outs || !n_out)
        return set_error(kInvalidArgument, "null argument");
    cudaStream_t st = opt.stream;
    const int64_t n = frame[0]->size;
    // filtered copy of the frame in temporaries, then the projection over it
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
    if (int e = process_filter(frame, ncols, filter_q, tp.data(), n_out, opt)) return e;
    std::vector<gdf_dtype> f(ncols);
    for (int c = 0; c < ncols; c++) f[c] = frame[c]->dtype;
    ProjectPlan pp = plan_project(project_q, f);
    if ((int)pp.columns.size() != n_outs) return set_error(kInvalidArgument, "out_columns count differs from the projection's");
    std::vector<gdf_column*> evald;
    for (size_t i = 0; i < pp.columns.size(); i++) {
        if (!pp.columns[i].first) continue;
        if (outs[i]->dtype != pp.eval_dtypes[pp.columns[i].second])
            return set_error(kInvalidArgument, "out column has the wrong dtype");
        outs[i]->size = *n_out;
        evald.push_back(outs[i]);
    }
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
    for (size_t i = 0, k = 0; i < pp.columns.size(); i++) {
        gdf_column* o = outs[i];
        if (pp.columns[i].first) {
            o->size = *n_out;
            o->null_count = (gdf_size_type)nulls[k++];
        } else {
            const gdf_column* src = tp[pp.columns[i].second];
            if (o->dtype != src->dtype) return set_error(kInvalidArgument, "out column has the wrong dtype");
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

}  // namespace ral
