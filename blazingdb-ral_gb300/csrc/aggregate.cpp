// aggregate.cpp — aggregations without GROUP BY whose inputs are expressions, fused with the
// reduction.
//
// Reference flow (src/operators/GroupBy.cpp): process_aggregate (:531-590) splits the
// LogicalAggregate into aggregations; compute_aggregations (:298-345) evaluates every input that
// contains an evaluation into a column of its own (evaluate_expression, a full pass writing n rows
// and their mask) and reduces it in aggregations_without_groupby (:231-296) with cudf::reduce.
// Here all evaluated inputs of the plan are ONE register program whose results are folded into
// the reductions inside the same kernel: each input column is read once and no intermediate
// column is written.
//
// Results follow the reference's flow exactly:
//   * output dtypes: get_aggregation_output_type (CalciteExpressionParsing.cpp:92-116): COUNT
//     INT64, SUM FLOAT64 for a float input else INT64, MIN / MAX the input's dtype, AVG FLOAT64;
//   * an evaluated column keeps null_count 0 (evaluate_expression leaves it, LogicalFilter.cpp:368),
//     and cudf's reduction consults a mask only when null_count > 0, so every row's value counts
//     and COUNT is the row count; a bare "$k" input keeps its null_count, its null rows are
//     skipped and COUNT is size - null_count; COUNT() reads column 0;
//   * SUM / MIN / MAX of an empty input, or of a bare input whose rows are all null, are null
//     scalars; AVG is null for an empty or all-null input, else the SUM as double divided by the
//     count (GroupBy.cpp:256-277);
//   * integer sums wrap in int64; float sums are exact IEEE adds in a fixed order (per thread,
//     then warps, blocks and block partials in index order), so a result does not change between
//     calls on the same GPU, but is not the bits of any one sequential order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "codegen.h"
#include "engine.h"
#include "frontend.h"
#include "jit.h"
#include "program.h"
#include "ral/ral_c.h"

namespace ral {

namespace {

gdf_dtype sum_type(gdf_dtype t) { return dtype_is_float(t) ? GDF_FLOAT64 : GDF_INT64; }

gdf_dtype aggregation_output_type(gdf_dtype in, int op) {
    switch (op) {
    case GDF_COUNT: return GDF_INT64;
    case GDF_SUM: return sum_type(in);
    case GDF_MIN: case GDF_MAX: return in;
    case GDF_AVG: return GDF_FLOAT64;
    default: return GDF_invalid;
    }
}

// A kernel result word (int64 bits or double bits, as the slot accumulates) as a scalar of `t`.
void set_scalar(gdf_scalar& s, gdf_dtype t, uint64_t word, bool float_acc) {
    std::memset(&s.data, 0, sizeof s.data);
    s.dtype = t;
    s.is_valid = true;
    double d;
    std::memcpy(&d, &word, 8);
    const int64_t i = (int64_t)word;
    switch (t) {
    case GDF_FLOAT64: { const double v = float_acc ? d : (double)i; std::memcpy(&s.data, &v, 8); break; }
    case GDF_FLOAT32: { const float v = (float)d; std::memcpy(&s.data, &v, 4); break; }
    case GDF_INT8: case GDF_BOOL8: { const int8_t v = (int8_t)i; std::memcpy(&s.data, &v, 1); break; }
    case GDF_INT16: { const int16_t v = (int16_t)i; std::memcpy(&s.data, &v, 2); break; }
    case GDF_INT32: case GDF_DATE32: case GDF_CATEGORY: case GDF_STRING_CATEGORY: {
        const int32_t v = (int32_t)i;
        std::memcpy(&s.data, &v, 4);
        break;
    }
    default: std::memcpy(&s.data, &i, 8); break;
    }
}

void set_null(gdf_scalar& s, gdf_dtype t) {
    std::memset(&s.data, 0, sizeof s.data);
    s.dtype = t;
    s.is_valid = false;
}

std::mutex g_agg_mu;
std::unordered_map<std::string, GeneratedKernel> g_agg_generated;

}  // namespace

// Everything the kernel needs, built on the host from the plan and the frame (no GPU calls).
struct AggregateBuild {
    AggregatePlan plan;
    Program prog;
    std::vector<ColumnDesc> bare;          // bare columns reduced by the kernel
    std::vector<int> bare_frame;           // their frame column numbers
    std::vector<AggregateSlot> slots;
    std::vector<int> slot_of;              // per aggregation: its kernel slot, or -1 (COUNT)
    std::vector<gdf_dtype> input_dtype;    // per aggregation: dtype of the reduced column
    Shape shape;
};

int build_aggregate(AggregateBuild& b, const std::vector<gdf_dtype>& dtypes, const std::vector<bool>& has_valid,
                    const std::vector<int64_t>& null_counts, const std::string& query) {
    b.plan = plan_aggregate(query, dtypes);
    if (!b.plan.group_columns.empty())
        return set_error(kUnsupported, "process_aggregate: GROUP BY aggregations are not on the expression path; "
                                       "only group=[{}] is supported");
    const auto& ap = b.plan;
    const int n_eval = (int)ap.eval_dtypes.size();
    if (n_eval > 0) {
        std::vector<ColumnDesc> ins;
        for (int c : ap.input_columns)
            ins.push_back(ColumnDesc{dtypes[c], (bool)has_valid[c], has_valid[c] && null_counts[c] != 0});
        std::vector<bool> out_valid(n_eval, false);  // the reduction does not read the evaluated masks
        std::string err;
        b.prog.float_literal_compat = config().float_literal_compat;
        const auto& pv = ap.pv;
        if (!b.prog.build(ins, ap.eval_dtypes, out_valid, pv.left.data(), pv.right.data(), pv.outs.data(),
                          (int)pv.left.size(), pv.final_pos.data(), pv.bops.data(), pv.uops.data(),
                          pv.lscalars.data(), pv.rscalars.data(), err))
            return set_error(kUnsupported, err);
    }
    std::unordered_map<int, int> bare_index;
    for (const auto& a : ap.aggregations) {
        const gdf_dtype in_t = a.evaluated ? ap.eval_dtypes[a.index] : dtypes[a.index];
        if (gdf_dtype_size(in_t) == 0) return set_error(kUnsupported, "process_aggregate: unsupported input dtype");
        b.input_dtype.push_back(in_t);
        if (a.op == GDF_COUNT) {
            b.slot_of.push_back(-1);
            continue;
        }
        AggregateSlot s;
        s.op = a.op == GDF_AVG ? GDF_SUM : a.op;
        s.evaluated = a.evaluated;
        s.dtype = in_t;
        if (a.evaluated) {
            s.index = a.index;
        } else {
            auto it = bare_index.find(a.index);
            if (it == bare_index.end()) {
                it = bare_index.emplace(a.index, (int)b.bare.size()).first;
                b.bare.push_back(ColumnDesc{dtypes[a.index], (bool)has_valid[a.index],
                                            has_valid[a.index] && null_counts[a.index] != 0});
                b.bare_frame.push_back(a.index);
            }
            s.index = it->second;
            s.skip_nulls = b.bare[s.index].nulls_possible;
        }
        b.slot_of.push_back((int)b.slots.size());
        b.slots.push_back(s);
    }
    int wb = 1;  // widest bare column: a lane's vector load of G elements is at most 16 bytes
    for (const auto& c : b.bare) wb = std::max(wb, gdf_dtype_size(c.dtype));
    if (n_eval > 0) {
        b.shape = eval_shape(b.prog);
        while (b.shape.G * wb > 16) {
            b.shape.G /= 2;
            b.shape.J *= 2;
        }
    } else {
        b.shape.G = std::max(1, 16 / wb);
        b.shape.J = 2;
        b.shape.threads = 512;
        b.shape.min_blocks = 2;
    }
    return kSuccess;
}

const GeneratedKernel& aggregate_kernel(const AggregateBuild& b) {
    const GeneratedKernel gk = generate_aggregate_kernel(b.prog, b.slots, b.bare, b.shape);
    std::lock_guard<std::mutex> lock(g_agg_mu);
    auto it = g_agg_generated.find(gk.name);
    if (it != g_agg_generated.end()) return it->second;
    return g_agg_generated.emplace(gk.name, gk).first->second;
}

int process_aggregate(gdf_column* const* frame, int n_cols, const char* query, gdf_scalar* results, int capacity,
                      int* num_results, cudaStream_t st) {
    if (!frame || n_cols <= 0 || !query || !num_results) return set_error(kInvalidArgument, "null argument");
    std::vector<gdf_dtype> dtypes(n_cols);
    std::vector<bool> has_valid(n_cols);
    std::vector<int64_t> nulls(n_cols);
    for (int c = 0; c < n_cols; c++) {
        if (!frame[c]) return set_error(kInvalidArgument, "null frame column");
        dtypes[c] = frame[c]->dtype;
        has_valid[c] = frame[c]->valid != nullptr;
        nulls[c] = frame[c]->null_count;
        if (frame[c]->valid && ((uintptr_t)frame[c]->valid & 3))
            return set_error(kInvalidArgument, "validity masks must be 4-byte aligned");
    }
    const int64_t n = frame[0]->size;
    for (int c = 1; c < n_cols; c++)
        if (frame[c]->size != n) return set_error(kInvalidArgument, "frame columns differ in size");
    CategoryScope categories(frame, n_cols);
    AggregateBuild b;
    if (int rc = build_aggregate(b, dtypes, has_valid, nulls, query)) return rc;
    const int n_agg = (int)b.plan.aggregations.size();
    *num_results = n_agg;
    if (!results || capacity < n_agg) return set_error(kInvalidArgument, "results array too small");
    const int S = (int)b.slots.size();

    std::vector<uint64_t> words(S, 0);
    if (S > 0 && n > 0) {
        Shape& s = b.shape;
        // vector loads need G-element alignment of every loaded column
        bool ok = true;
        const auto ref = b.prog.n_out > 0 ? b.prog.inputs_referenced() : std::vector<bool>();
        for (size_t k = 0; k < b.plan.input_columns.size(); k++)
            if (ref[k] && ((uintptr_t)frame[b.plan.input_columns[k]]->data % ((size_t)s.G * gdf_dtype_size(dtypes[b.plan.input_columns[k]]))))
                ok = false;
        for (size_t k = 0; k < b.bare.size(); k++)
            if ((uintptr_t)frame[b.bare_frame[k]]->data % ((size_t)s.G * gdf_dtype_size(b.bare[k].dtype))) ok = false;
        if (!ok) { s.G = 1; s.J = 4; }
        for (int c = 0; c < n_cols; c++)
            if (!frame[c]->data) return set_error(kInvalidArgument, "frame column without data");
        const GeneratedKernel& gk = aggregate_kernel(b);
        std::string err;
        const CompiledKernel* k = jit_get(gk, err);
        if (!k) return set_error(kJitError, err);
        const ParamLayout& L = k->layout;
        const int64_t rows_per_block = (int64_t)32 * s.G * s.J * (s.threads / 32);
        const int grid = launch_blocks(*k, s.threads, rows_per_block, n);
        const int64_t nwords = aggregate_scratch_words(S, grid);
        uint64_t* d = nullptr;
        if (int e = check_cuda(cudaMallocAsync((void**)&d, (size_t)nwords * 8, st), "cudaMallocAsync")) return e;
        int rc = check_cuda(cudaMemsetAsync(d, 0, (size_t)nwords * 8, st), "cudaMemsetAsync");
        std::vector<uint64_t> slots(L.total, 0);
        slots[L.n_rows] = (uint64_t)n;
        for (size_t c = 0; c < b.plan.input_columns.size(); c++) {
            slots[L.in_data + c] = (uint64_t)(uintptr_t)frame[b.plan.input_columns[c]]->data;
            slots[L.in_valid + c] = (uint64_t)(uintptr_t)frame[b.plan.input_columns[c]]->valid;
        }
        slots[L.counts + 1] = (uint64_t)(uintptr_t)d;
        const int NB = (int)b.bare.size();
        for (int c = 0; c < NB; c++) {
            slots[L.counts + 2 + c] = (uint64_t)(uintptr_t)frame[b.bare_frame[c]]->data;
            slots[L.counts + 2 + NB + c] = (uint64_t)(uintptr_t)frame[b.bare_frame[c]]->valid;
        }
        fill_scalars(b.prog, L, slots);
        if (!rc) {
            void* args[] = {slots.data()};
            rc = check_cuda(cudaLaunchKernel((const void*)k->kernel, dim3(grid), dim3(s.threads), args, 0, st),
                            "launch of the aggregate kernel");
            if (!rc) note_launch();
        }
        if (!rc) rc = check_cuda(cudaMemcpyAsync(words.data(), d + 1, (size_t)S * 8, cudaMemcpyDeviceToHost, st),
                                 "cudaMemcpyAsync");
        cudaFreeAsync(d, st);
        if (int e = check_cuda(cudaStreamSynchronize(st), "process_aggregate")) return e;
        if (rc) return rc;
    }

    for (int i = 0; i < n_agg; i++) {
        const auto& a = b.plan.aggregations[i];
        const gdf_dtype in_t = b.input_dtype[i];
        const gdf_dtype out_t = aggregation_output_type(in_t, a.op);
        // rows the reduction counts: every row of an evaluated column (null_count 0), the non-null
        // rows of a bare column
        const int64_t count = a.evaluated ? n : n - (int64_t)frame[a.index]->null_count;
        gdf_scalar& r = results[i];
        if (a.op == GDF_COUNT) {
            set_scalar(r, GDF_INT64, (uint64_t)count, false);
            continue;
        }
        if (n == 0 || count <= 0) {  // empty, or every row null: cudf returns an invalid scalar
            set_null(r, out_t);
            continue;
        }
        const uint64_t w = words[b.slot_of[i]];
        const bool facc = dtype_is_float(in_t);
        if (a.op == GDF_AVG) {
            double sum;
            if (facc) std::memcpy(&sum, &w, 8);
            else sum = (double)(int64_t)w;
            const double avg = sum / (double)count;
            uint64_t bits;
            std::memcpy(&bits, &avg, 8);
            set_scalar(r, GDF_FLOAT64, bits, true);
        } else {
            set_scalar(r, out_t, w, facc);
        }
    }
    return kSuccess;
}

int aggregate_source(const gdf_dtype* dtypes, const int32_t* nullable, const int64_t* null_counts, int n_cols,
                     const char* query, bool compile, std::string& source, std::string& log) {
    std::vector<gdf_dtype> dt(dtypes, dtypes + n_cols);
    std::vector<bool> hv(n_cols);
    std::vector<int64_t> nc(n_cols);
    for (int c = 0; c < n_cols; c++) {
        hv[c] = nullable && nullable[c] != 0;
        nc[c] = null_counts ? null_counts[c] : (hv[c] ? 1 : 0);
    }
    AggregateBuild b;
    if (int rc = build_aggregate(b, dt, hv, nc, query)) return rc;
    if (b.slots.empty()) {
        source.clear();
        return kSuccess;
    }
    const GeneratedKernel& gk = aggregate_kernel(b);
    source = gk.source;
    if (compile) {
        std::string err;
        size_t bytes = 0;
        if (!jit_compile_only(gk, &bytes, &log, err)) return set_error(kJitError, err);
    }
    return kSuccess;
}

}  // namespace ral
