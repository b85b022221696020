// capi.cpp — the extern "C" entry points declared in include/ral/ral_c.h and include/ral/ral_debug.h.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "batch.h"
#include "codegen.h"
#include "engine.h"
#include "filter.h"
#include "frontend.h"
#include "jit.h"
#include "kernels.h"
#include "server.h"
#include "ral/ral_c.h"
#include "textscan.h"
#include "ral/ral_debug.h"

using namespace ral;

namespace ral {
int softfp_selftest(long long n, unsigned long long seed, long long* counts, unsigned long long* first_operands);
}

namespace {

template <typename F>
int guarded(F&& f) {
    try {
        return f();
    } catch (const ParseError& e) {
        return set_error(kParseError, e.what());
    } catch (const std::exception& e) {
        return set_error(kInvalidArgument, e.what());
    }
}

void copy_out(const std::string& s, char* buf, int64_t cap) {
    if (!buf || cap <= 0) return;
    size_t n = std::min<size_t>(s.size(), (size_t)cap - 1);
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
}

int count_nulls(gdf_column* col, cudaStream_t st) {
    if (col->size == 0 || col->valid == nullptr) {
        col->null_count = 0;
        return kSuccess;
    }
    unsigned long long* d = nullptr;
    if (int e = check_cuda(cudaMallocAsync((void**)&d, sizeof(unsigned long long), st), "cudaMallocAsync")) return e;
    cudaMemsetAsync(d, 0, sizeof(unsigned long long), st);
    if (int e = check_cuda(launch_count_valid((const uint32_t*)col->valid, col->size, d, st), "count_valid")) return e;
    unsigned long long h = 0;
    cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (int e = check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return e;
    col->null_count = (gdf_size_type)(col->size - (int64_t)h);
    return kSuccess;
}

}  // namespace

extern "C" {

const char* ral_last_error(void) { return last_error(); }
const char* ral_version(void) { return "ralgpu 0.1 (sm_103a)"; }

int ral_perform_operation(gdf_column* const* output_columns, int32_t num_outputs, gdf_column* const* input_columns,
                          int32_t num_inputs, const column_index_type* left_inputs,
                          const column_index_type* right_inputs, const column_index_type* outputs,
                          int32_t num_operations, const column_index_type* final_output_positions,
                          const int32_t* operators, const int32_t* unary_operators, const gdf_scalar* left_scalars,
                          const gdf_scalar* right_scalars, const column_index_type* new_input_indices,
                          int32_t num_new_input_indices) {
    (void)new_input_indices;
    (void)num_new_input_indices;
    return guarded([&] {
        ProgramArrays pa{left_inputs, right_inputs, outputs, num_operations, final_output_positions,
                         operators, unary_operators, left_scalars, right_scalars};
        EvalOptions opt;
        opt.stream = cudaStreamPerThread;
        opt.sync = true;
        return perform_operation(output_columns, num_outputs, input_columns, num_inputs, pa, opt);
    });
}

int ral_perform_operation_host(gdf_column* const* output_columns, int32_t num_outputs, gdf_column* const* input_columns,
                               int32_t num_inputs, const column_index_type* left_inputs,
                               const column_index_type* right_inputs, const column_index_type* outputs,
                               int32_t num_operations, const column_index_type* final_output_positions,
                               const int32_t* operators, const int32_t* unary_operators, const gdf_scalar* left_scalars,
                               const gdf_scalar* right_scalars, int64_t chunk_rows) {
    return guarded([&] {
        ProgramArrays pa{left_inputs, right_inputs, outputs, num_operations, final_output_positions,
                         operators, unary_operators, left_scalars, right_scalars};
        return perform_operation_host(output_columns, num_outputs, input_columns, num_inputs, pa, chunk_rows);
    });
}

int ral_perform_operation_async(gdf_column* const* output_columns, int32_t num_outputs,
                                gdf_column* const* input_columns, int32_t num_inputs,
                                const column_index_type* left_inputs, const column_index_type* right_inputs,
                                const column_index_type* outputs, int32_t num_operations,
                                const column_index_type* final_output_positions, const int32_t* operators,
                                const int32_t* unary_operators, const gdf_scalar* left_scalars,
                                const gdf_scalar* right_scalars, void* stream, int64_t* null_counts) {
    return guarded([&] {
        ProgramArrays pa{left_inputs, right_inputs, outputs, num_operations, final_output_positions,
                         operators, unary_operators, left_scalars, right_scalars};
        EvalOptions opt;
        opt.stream = (cudaStream_t)stream;
        opt.sync = false;
        opt.null_counts = null_counts;
        return perform_operation(output_columns, num_outputs, input_columns, num_inputs, pa, opt);
    });
}

int ral_evaluate_expression(gdf_column* const* frame, int32_t num_columns, const char* expression,
                            gdf_column* output) {
    return guarded([&] {
        if (!frame || num_columns <= 0 || !expression || !output)
            return set_error(kInvalidArgument, "evaluate_expression: null argument");
        CategoryScope categories(frame, num_columns);
        ExpressionPlan ep = plan_expression(expression, num_columns);
        cudaStream_t st = cudaStreamPerThread;
        if (ep.clone) {
            const gdf_column* src = frame[ep.clone_column];
            if (src->dtype != output->dtype)
                return set_error(kInvalidArgument, "evaluate_expression: \"$k\" output must have column k's dtype");
            if (output->size < src->size) return set_error(kInvalidArgument, "evaluate_expression: output too small");
            const size_t bytes = (size_t)src->size * gdf_dtype_size(src->dtype);
            if (bytes) cudaMemcpyAsync(output->data, src->data, bytes, cudaMemcpyDeviceToDevice, st);
            if (src->valid && output->valid) {
                cudaMemcpyAsync(output->valid, src->valid, (src->size + 7) / 8, cudaMemcpyDeviceToDevice, st);
            } else if (output->valid) {
                cudaMemsetAsync(output->valid, 0xFF, (src->size + 7) / 8, st);
            }
            output->null_count = src->null_count;
            return check_cuda(cudaStreamSynchronize(st), "evaluate_expression clone");
        }
        std::vector<gdf_column*> ins;
        for (int c : ep.input_columns) ins.push_back(frame[c]);
        gdf_column* outs[1] = {output};
        ProgramArrays pa{ep.pv.left.data(), ep.pv.right.data(), ep.pv.outs.data(), (int32_t)ep.pv.left.size(),
                         ep.pv.final_pos.data(), ep.pv.bops.data(), ep.pv.uops.data(), ep.pv.lscalars.data(),
                         ep.pv.rscalars.data()};
        EvalOptions opt;
        opt.stream = st;
        return perform_operation(outs, 1, ins.data(), (int)ins.size(), pa, opt);
    });
}

int ral_add_expression_to_plan(const char* expression, column_index_type expression_position,
                               column_index_type num_outputs, column_index_type num_inputs,
                               const column_index_type* new_input_indices, int32_t num_frame_columns,
                               column_index_type* left_inputs, column_index_type* right_inputs,
                               column_index_type* outputs, int32_t* operators, int32_t* unary_operators,
                               gdf_scalar* left_scalars, gdf_scalar* right_scalars, int32_t* num_operations,
                               int32_t capacity) {
    return guarded([&] {
        if (!expression || !num_operations) return set_error(kInvalidArgument, "null argument");
        auto e = parse_expression(expression);
        std::vector<int> remap(new_input_indices, new_input_indices + num_frame_columns);
        ProgramVectors pv;
        emit_expression(*e, expression_position, num_outputs, num_inputs, remap, pv);
        const int base = *num_operations;
        if (base + (int)pv.left.size() > capacity) return set_error(kInvalidArgument, "capacity too small");
        for (size_t k = 0; k < pv.left.size(); k++) {
            left_inputs[base + k] = pv.left[k];
            right_inputs[base + k] = pv.right[k];
            outputs[base + k] = pv.outs[k];
            operators[base + k] = pv.bops[k];
            unary_operators[base + k] = pv.uops[k];
            left_scalars[base + k] = pv.lscalars[k];
            right_scalars[base + k] = pv.rscalars[k];
        }
        *num_operations = base + (int)pv.left.size();
        return (int)kSuccess;
    });
}

int ral_get_output_type_expression(const gdf_dtype* frame_dtypes, int32_t num_columns, const char* expression,
                                   gdf_dtype* dtype_out) {
    return guarded([&] {
        auto e = parse_expression(expression);
        std::vector<gdf_dtype> f(frame_dtypes, frame_dtypes + num_columns);
        *dtype_out = expression_output_type(*e, f);
        return (int)kSuccess;
    });
}

int ral_project_output_types(const gdf_dtype* frame_dtypes, int32_t num_columns, const char* query_part,
                             int32_t* num_projected, gdf_dtype* dtypes_out, int32_t* is_evaluated_out,
                             int32_t capacity) {
    return guarded([&] {
        std::vector<gdf_dtype> f(frame_dtypes, frame_dtypes + num_columns);
        TypesOnlyScope types_only;
        ProjectPlan pp = plan_project(query_part, f);
        *num_projected = (int32_t)pp.columns.size();
        if ((int)pp.columns.size() > capacity) return set_error(kInvalidArgument, "capacity too small");
        for (size_t i = 0; i < pp.columns.size(); i++) {
            is_evaluated_out[i] = pp.columns[i].first ? 1 : 0;
            dtypes_out[i] = pp.columns[i].first ? pp.eval_dtypes[pp.columns[i].second] : f[pp.columns[i].second];
        }
        return (int)kSuccess;
    });
}

int ral_parse_project_plan(const gdf_dtype* frame_dtypes, int32_t num_columns, const char* query_part,
                           int32_t capacity_ops, int32_t capacity_cols, int32_t* num_input_columns,
                           int32_t* input_columns, int32_t* num_evaluated, gdf_dtype* evaluated_dtypes,
                           int32_t* num_operations, column_index_type* left_inputs, column_index_type* right_inputs,
                           column_index_type* outputs, column_index_type* final_output_positions,
                           int32_t* operators, int32_t* unary_operators, gdf_scalar* left_scalars,
                           gdf_scalar* right_scalars) {
    return guarded([&] {
        std::vector<gdf_dtype> f(frame_dtypes, frame_dtypes + num_columns);
        ProjectPlan pp = plan_project(query_part, f);
        const int nops = (int)pp.pv.left.size();
        if (nops > capacity_ops || (int)pp.input_columns.size() > capacity_cols || (int)pp.eval_dtypes.size() > capacity_cols)
            return set_error(kInvalidArgument, "capacity too small");
        *num_input_columns = (int32_t)pp.input_columns.size();
        for (size_t i = 0; i < pp.input_columns.size(); i++) input_columns[i] = pp.input_columns[i];
        *num_evaluated = (int32_t)pp.eval_dtypes.size();
        for (size_t i = 0; i < pp.eval_dtypes.size(); i++) {
            evaluated_dtypes[i] = pp.eval_dtypes[i];
            final_output_positions[i] = pp.pv.final_pos[i];
        }
        *num_operations = nops;
        for (int k = 0; k < nops; k++) {
            left_inputs[k] = pp.pv.left[k];
            right_inputs[k] = pp.pv.right[k];
            outputs[k] = pp.pv.outs[k];
            operators[k] = pp.pv.bops[k];
            unary_operators[k] = pp.pv.uops[k];
            left_scalars[k] = pp.pv.lscalars[k];
            right_scalars[k] = pp.pv.rscalars[k];
        }
        return (int)kSuccess;
    });
}

int ral_batch_debug_source(const ral_batch* batch, int32_t compile, char* source_out, int64_t source_capacity,
                           char* log_out, int64_t log_capacity);

int ral_execute_project_plan(gdf_column* const* frame, int32_t num_columns, const char* query_part,
                             gdf_column* const* out_columns, int32_t num_out_columns) {
    return guarded([&] {
        std::vector<gdf_dtype> f(num_columns);
        for (int c = 0; c < num_columns; c++) f[c] = frame[c]->dtype;
        CategoryScope categories(frame, num_columns);
        ProjectPlan pp = plan_project(query_part, f);
        if ((int)pp.columns.size() != num_out_columns)
            return set_error(kInvalidArgument, "out_columns count differs from the projection's");
        cudaStream_t st = cudaStreamPerThread;
        const int64_t n = frame[0]->size;
        std::vector<gdf_column*> evald;
        for (size_t i = 0; i < pp.columns.size(); i++) {
            if (!pp.columns[i].first) continue;
            gdf_column* o = out_columns[i];
            if (o->dtype != pp.eval_dtypes[pp.columns[i].second])
                return set_error(kInvalidArgument, "out column " + std::to_string(i) + " has the wrong dtype");
            evald.push_back(o);
        }
        std::vector<int64_t> nulls(evald.size(), 0);
        if (!evald.empty()) {
            std::vector<gdf_column*> ins;
            for (int c : pp.input_columns) ins.push_back(frame[c]);
            ProgramArrays pa{pp.pv.left.data(), pp.pv.right.data(), pp.pv.outs.data(), (int32_t)pp.pv.left.size(),
                             pp.pv.final_pos.data(), pp.pv.bops.data(), pp.pv.uops.data(), pp.pv.lscalars.data(),
                             pp.pv.rscalars.data()};
            EvalOptions opt;
            opt.stream = st;
            opt.null_counts = nulls.data();
            if (int e = perform_operation(evald.data(), (int)evald.size(), ins.data(), (int)ins.size(), pa, opt)) return e;
        }
        for (size_t i = 0, k = 0; i < pp.columns.size(); i++) {
            gdf_column* o = out_columns[i];
            if (pp.columns[i].first) {
                o->size = (gdf_size_type)n;
                o->null_count = (gdf_size_type)nulls[k++];
            } else {
                *o = *frame[pp.columns[i].second];
                if (int e = count_nulls(o, st)) return e;
                frame[pp.columns[i].second]->null_count = o->null_count;
            }
        }
        return (int)kSuccess;
    });
}

int ral_materialize_column(const gdf_column* input, gdf_column* output, const gdf_column* row_indices) {
    return guarded([&] {
        if (!input || !output || !row_indices) return set_error(kInvalidArgument, "null argument");
        const int w = gdf_dtype_size(input->dtype);
        const int iw = gdf_dtype_size(row_indices->dtype);
        if (w == 0 || iw == 0 || dtype_is_float(row_indices->dtype))
            return set_error(kInvalidArgument, "materialize_column: unsupported dtype");
        if (gdf_dtype_size(output->dtype) != w) return set_error(kInvalidArgument, "materialize_column: width mismatch");
        const int64_t n = row_indices->size;
        cudaStream_t st = cudaStreamPerThread;
        unsigned long long* d = nullptr;
        if (output->valid) {
            if (int e = check_cuda(cudaMallocAsync((void**)&d, sizeof(unsigned long long), st), "cudaMallocAsync")) return e;
            cudaMemsetAsync(d, 0, sizeof(unsigned long long), st);
        }
        if (int e = check_cuda(launch_gather(w, input->data, (const uint32_t*)input->valid, input->size, row_indices->data, iw, n,
                                             output->data, (uint32_t*)output->valid, d, st),
                               "gather"))
            return e;
        unsigned long long h = 0;
        if (d) {
            cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, st);
            cudaFreeAsync(d, st);
        }
        if (int e = check_cuda(cudaStreamSynchronize(st), "materialize_column")) return e;
        output->size = (gdf_size_type)n;
        output->null_count = output->valid ? (gdf_size_type)(n - (int64_t)h) : 0;
        return (int)kSuccess;
    });
}

int ral_text_scan_rows(const char* data, int64_t n_bytes, char line_terminator, int32_t skip_rows, int64_t* rows) {
    return guarded([&] { return text_scan_rows(data, n_bytes, line_terminator, skip_rows, rows); });
}

int ral_text_scan_filter(const char* data, int64_t n_bytes, char delimiter, char line_terminator, int32_t skip_rows,
                         const int32_t* file_dtypes, int32_t n_file_columns, const int32_t* projections,
                         int32_t n_projections, const char* filter_query_part, gdf_column* const* out_columns,
                         gdf_size_type* num_rows_out) {
    return guarded([&] {
        return text_scan_filter(data, n_bytes, delimiter, line_terminator, skip_rows, file_dtypes, n_file_columns,
                                projections, n_projections, filter_query_part, out_columns, num_rows_out);
    });
}

int ral_text_scan_filter_host(const char* text, int64_t n_bytes, char delimiter, char line_terminator,
                              int32_t skip_rows, const int32_t* file_dtypes, int32_t n_file_columns,
                              const int32_t* projections, int32_t n_projections, const char* filter_query_part,
                              gdf_column* const* out_columns, gdf_size_type* num_rows_out) {
    return guarded([&] {
        return text_scan_filter_host(text, n_bytes, delimiter, line_terminator, skip_rows, file_dtypes, n_file_columns,
                                     projections, n_projections, filter_query_part, out_columns, num_rows_out);
    });
}

int ral_parquet_schema(const uint8_t* file, int64_t n_bytes, int64_t* rows, int32_t* n_columns, int32_t* dtypes,
                       int32_t capacity) {
    return guarded([&] { return parquet_schema(file, n_bytes, rows, n_columns, dtypes, capacity); });
}

int ral_parquet_scan_filter(const uint8_t* file, int64_t n_bytes, const int32_t* projections, int32_t n_projections,
                            const char* filter_query_part, gdf_column* const* out_columns, gdf_size_type* num_rows_out) {
    return guarded([&] {
        return parquet_scan_filter(file, n_bytes, projections, n_projections, filter_query_part, out_columns, num_rows_out);
    });
}

int ral_materialize_columns(const gdf_column* const* inputs, gdf_column* const* outputs, int32_t num_columns,
                            const gdf_column* row_indices) {
    return guarded([&] {
        if (!row_indices || (num_columns > 0 && (!inputs || !outputs))) return set_error(kInvalidArgument, "null argument");
        if (num_columns < 0 || num_columns > kMaxGatherColumns)
            return set_error(kInvalidArgument, "materialize_columns: 0.." + std::to_string(kMaxGatherColumns) + " columns");
        const int iw = gdf_dtype_size(row_indices->dtype);
        if (iw == 0 || dtype_is_float(row_indices->dtype))
            return set_error(kInvalidArgument, "materialize_columns: row_indices must be an INT8/16/32/64 column");
        const int64_t n = row_indices->size;
        if (n < 0) return set_error(kInvalidArgument, "materialize_columns: negative row count");
        if (n > 0 && !row_indices->data) return set_error(kInvalidArgument, "materialize_columns: row_indices without data");
        GatherColumnsParams p{};
        p.idx = row_indices->data;
        p.idx_width = iw;
        p.n_out = n;
        p.num_columns = num_columns;
        int64_t n_in = -1;
        for (int c = 0; c < num_columns; c++) {
            const gdf_column* in = inputs[c];
            gdf_column* out = outputs[c];
            if (!in || !out) return set_error(kInvalidArgument, "materialize_columns: null column");
            const int w = gdf_dtype_size(in->dtype);
            if (w == 0) return set_error(kInvalidArgument, "materialize_columns: unsupported dtype of column " + std::to_string(c));
            if (gdf_dtype_size(out->dtype) != w)
                return set_error(kInvalidArgument, "materialize_columns: width mismatch in column " + std::to_string(c));
            if (n_in < 0) n_in = in->size;
            if (in->size != n_in) return set_error(kInvalidArgument, "materialize_columns: input columns differ in size");
            if (n > 0 && ((in->size > 0 && !in->data) || !out->data))
                return set_error(kInvalidArgument, "materialize_columns: column without data");
            if (((uintptr_t)in->valid & 3) || ((uintptr_t)out->valid & 3))
                return set_error(kInvalidArgument, "materialize_columns: masks must be 4-byte aligned");
            p.col[c] = GatherColumn{in->data, (const uint32_t*)in->valid, out->data, (uint32_t*)out->valid, w, 0};
        }
        p.n_in = n_in < 0 ? 0 : n_in;
        cudaStream_t st = cudaStreamPerThread;
        std::vector<unsigned long long> h(num_columns > 0 ? num_columns : 1, 0);
        if (n > 0 && num_columns > 0) {
            unsigned long long* d = nullptr;
            if (int e = check_cuda(cudaMallocAsync((void**)&d, sizeof(unsigned long long) * num_columns, st), "cudaMallocAsync")) return e;
            int rc = check_cuda(cudaMemsetAsync(d, 0, sizeof(unsigned long long) * num_columns, st), "cudaMemsetAsync");
            p.valid_counts = d;
            if (!rc) rc = check_cuda(launch_gather_columns(p, st), "gather_columns");
            if (!rc) rc = check_cuda(cudaMemcpyAsync(h.data(), d, sizeof(unsigned long long) * num_columns,
                                                     cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
            cudaFreeAsync(d, st);
            if (int e = check_cuda(cudaStreamSynchronize(st), "materialize_columns")) return e;
            if (rc) return rc;
        }
        for (int c = 0; c < num_columns; c++) {
            outputs[c]->size = (gdf_size_type)n;
            outputs[c]->null_count = outputs[c]->valid ? (gdf_size_type)(n - (int64_t)h[c]) : 0;
        }
        return (int)kSuccess;
    });
}

int ral_process_aggregate(gdf_column* const* frame_columns, int32_t num_columns, const char* query_part,
                          gdf_scalar* results, int32_t capacity, int32_t* num_results) {
    return guarded([&] {
        int n = 0;
        const int rc = process_aggregate(frame_columns, num_columns, query_part, results, capacity, &n,
                                         cudaStreamPerThread);
        if (num_results) *num_results = n;
        return rc;
    });
}

int ral_debug_aggregate_source(const gdf_dtype* frame_dtypes, const int32_t* frame_nullable,
                               const int64_t* frame_null_counts, int32_t num_columns, const char* query_part,
                               int32_t compile, char* source_out, int64_t source_capacity, char* log_out,
                               int64_t log_capacity) {
    return guarded([&] {
        if (!frame_dtypes || num_columns <= 0 || !query_part) return set_error(kInvalidArgument, "null argument");
        std::string src, log;
        const int rc = aggregate_source(frame_dtypes, frame_nullable, frame_null_counts, num_columns, query_part,
                                        compile != 0, src, log);
        copy_out(src, source_out, source_capacity);
        copy_out(log, log_out, log_capacity);
        return rc;
    });
}

int ral_filter_project_host(gdf_column* const* frame_columns, int32_t num_columns, const char* filter_query_part,
                            const char* project_query_part, gdf_column* const* out_columns, int32_t num_out_columns,
                            gdf_size_type* num_rows_out, int64_t chunk_rows) {
    return guarded([&] {
        return filter_host(frame_columns, num_columns, filter_query_part, project_query_part, out_columns,
                           num_out_columns, num_rows_out, chunk_rows);
    });
}

int ral_debug_call_timing(int32_t enable, int32_t reset, int64_t* calls, double* us4) {
    return call_timing_query(enable != 0, reset != 0, calls, us4);
}

int ral_debug_text_scan_source(const int32_t* file_dtypes, int32_t n_file_columns, const int32_t* projections,
                               int32_t n_projections, const char* filter_query_part, int32_t compile, char* source_out,
                               int64_t source_capacity, char* log_out, int64_t log_capacity) {
    return guarded([&] {
        std::string src, log;
        const int rc = text_scan_source(file_dtypes, n_file_columns, projections, n_projections, filter_query_part,
                                        compile != 0, src, log);
        copy_out(src, source_out, source_capacity);
        copy_out(log, log_out, log_capacity);
        return rc;
    });
}

int ral_debug_filter_grid_launches(int64_t* launches) {
    if (!launches) return set_error(kInvalidArgument, "null argument");
    *launches = filter_grid_launches();
    return kSuccess;
}

int ral_apply_boolean_mask(const gdf_column* stencil, gdf_column* out_indices, gdf_size_type* num_rows_out) {
    return guarded([&] {
        if (!stencil || !out_indices || !num_rows_out) return set_error(kInvalidArgument, "null argument");
        if (gdf_dtype_size(stencil->dtype) != 1) return set_error(kInvalidArgument, "stencil must be INT8 or BOOL8");
        if (out_indices->dtype != GDF_INT32) return set_error(kInvalidArgument, "out_indices must be INT32");
        if (stencil->valid && ((uintptr_t)stencil->valid & 3)) return set_error(kInvalidArgument, "mask must be 4-byte aligned");
        const int64_t n = stencil->size;
        if (n == 0) {
            out_indices->size = 0;
            *num_rows_out = 0;
            return (int)kSuccess;
        }
        if (!stencil->data || !out_indices->data) return set_error(kInvalidArgument, "column without data");
        cudaStream_t st = cudaStreamPerThread;
        const int64_t words = compact_scratch_words(n);
        unsigned long long* scratch = nullptr;
        if (int e = check_cuda(cudaMallocAsync((void**)&scratch, (size_t)words * 8, st), "cudaMallocAsync")) return e;
        if (int e = check_cuda(cudaMemsetAsync(scratch, 0, (size_t)words * 8, st), "cudaMemsetAsync")) {
            cudaFreeAsync(scratch, st);
            return e;
        }
        int rc = check_cuda(launch_compact_stencil((const int8_t*)stencil->data, (const uint32_t*)stencil->valid, n,
                                                   (int32_t*)out_indices->data, scratch, st),
                            "compaction");
        unsigned long long h[3] = {0, 0, 0};
        if (rc == kSuccess) cudaMemcpyAsync(h, scratch, sizeof h, cudaMemcpyDeviceToHost, st);
        cudaFreeAsync(scratch, st);
        if (int e = check_cuda(cudaStreamSynchronize(st), "apply_boolean_mask")) return e;
        if (rc) return rc;
        if (h[1]) return set_error(kTimeout, "compaction look-back wait gave up");
        out_indices->size = (gdf_size_type)h[2];
        *num_rows_out = (gdf_size_type)h[2];
        return (int)kSuccess;
    });
}

int ral_process_filter(gdf_column* const* frame, int32_t num_columns, const char* query_part,
                       gdf_column* const* out_columns, gdf_size_type* num_rows_out) {
    return guarded([&] {
        FilterOptions opt;
        opt.stream = cudaStreamPerThread;
        opt.sync = true;
        return process_filter(frame, num_columns, query_part, out_columns, num_rows_out, opt);
    });
}

int ral_process_filter_async(gdf_column* const* frame, int32_t num_columns, const char* query_part,
                             gdf_column* const* out_columns, gdf_size_type* num_rows_out, void* stream) {
    return guarded([&] {
        FilterOptions opt;
        opt.stream = (cudaStream_t)stream;
        opt.sync = true;
        return process_filter(frame, num_columns, query_part, out_columns, num_rows_out, opt);
    });
}

int ral_filter_project(gdf_column* const* frame, int32_t num_columns, const char* filter_query_part,
                       const char* project_query_part, gdf_column* const* out_columns, int32_t num_out_columns,
                       gdf_size_type* num_rows_out) {
    return guarded([&] {
        FilterOptions opt;
        opt.stream = cudaStreamPerThread;
        opt.sync = true;
        return filter_project(frame, num_columns, filter_query_part, project_query_part, out_columns,
                              num_out_columns, num_rows_out, opt);
    });
}

int ral_debug_program_source(const gdf_dtype* input_dtypes, const int32_t* input_nullable, int32_t num_inputs,
                             const gdf_dtype* output_dtypes, const int32_t* output_nullable, int32_t num_outputs,
                             const column_index_type* left_inputs, const column_index_type* right_inputs,
                             const column_index_type* outputs, int32_t num_operations,
                             const column_index_type* final_output_positions, const int32_t* operators,
                             const int32_t* unary_operators, const gdf_scalar* left_scalars,
                             const gdf_scalar* right_scalars, int32_t compile, char* source_out,
                             int64_t source_capacity, char* log_out, int64_t log_capacity) {
    return guarded([&] {
        std::vector<ColumnDesc> ins(num_inputs);
        for (int c = 0; c < num_inputs; c++) {
            ins[c].dtype = input_dtypes[c];
            ins[c].has_valid = input_nullable[c] != 0;
            ins[c].nulls_possible = input_nullable[c] != 0;
        }
        std::vector<gdf_dtype> ot(output_dtypes, output_dtypes + num_outputs);
        std::vector<bool> ov(num_outputs);
        for (int o = 0; o < num_outputs; o++) ov[o] = output_nullable[o] != 0;
        Program p;
        std::string err;
        if (!p.build(ins, ot, ov, left_inputs, right_inputs, outputs, num_operations, final_output_positions,
                     operators, unary_operators, left_scalars, right_scalars, err))
            return set_error(kUnsupported, err);
        GeneratedKernel gk = generate_eval_kernel(p, eval_shape(p));
        copy_out(std::string(jit_prelude()) + "\n" + gk.source, source_out, source_capacity);
        if (compile) {
            size_t bytes = 0;
            std::string log;
            if (!jit_compile_only(gk, &bytes, &log, err)) {
                copy_out(err, log_out, log_capacity);
                return set_error(kJitError, err);
            }
            copy_out(log, log_out, log_capacity);
        }
        return (int)kSuccess;
    });
}

int ral_debug_filter_source(const gdf_dtype* frame_dtypes, const int32_t* frame_nullable, int32_t num_columns,
                            const char* filter_query_part, const char* project_query_part, int32_t compile,
                            char* source_out, int64_t source_capacity, char* log_out, int64_t log_capacity) {
    return guarded([&] {
        std::vector<gdf_column> cols(num_columns);
        std::vector<gdf_column*> ptrs(num_columns);
        for (int c = 0; c < num_columns; c++) {
            cols[c] = gdf_column{};
            cols[c].dtype = frame_dtypes[c];
            cols[c].valid = frame_nullable[c] ? (gdf_valid_type*)(uintptr_t)64 : nullptr;
            cols[c].null_count = frame_nullable[c] ? 1 : 0;
            ptrs[c] = &cols[c];
        }
        std::string src, log;
        int rc = debug_filter_source(ptrs.data(), num_columns, filter_query_part, project_query_part, compile != 0, src, log);
        copy_out(src, source_out, source_capacity);
        copy_out(log, log_out, log_capacity);
        return rc;
    });
}

struct ral_server_s {
    ral::Server s;
    ral_server_s(size_t b, int w, int m, int64_t r) : s(b, w, m, r) {}
};

struct ral_batch_s {
    ral::Batch b;
};

int ral_batch_create(ral_batch** batch) {
    return guarded([&] {
        if (!batch) return set_error(kInvalidArgument, "null argument");
        *batch = new ral_batch_s();
        return (int)kSuccess;
    });
}

int ral_batch_add(ral_batch* batch, gdf_column* const* output_columns, int32_t num_outputs,
                  gdf_column* const* input_columns, int32_t num_inputs, const column_index_type* left_inputs,
                  const column_index_type* right_inputs, const column_index_type* outputs, int32_t num_operations,
                  const column_index_type* final_output_positions, const int32_t* operators,
                  const int32_t* unary_operators, const gdf_scalar* left_scalars, const gdf_scalar* right_scalars,
                  int32_t* program_index) {
    return guarded([&] {
        if (!batch) return set_error(kInvalidArgument, "null batch");
        ProgramArrays pa{left_inputs, right_inputs, outputs, num_operations, final_output_positions,
                         operators, unary_operators, left_scalars, right_scalars};
        const int idx = batch->b.add(output_columns, num_outputs, input_columns, num_inputs, pa);
        if (idx < 0) return -idx;
        if (program_index) *program_index = idx;
        return (int)kSuccess;
    });
}

int ral_batch_prepare(ral_batch* batch) {
    return guarded([&] {
        if (!batch) return set_error(kInvalidArgument, "null batch");
        return batch->b.prepare(cudaStreamPerThread);
    });
}

int ral_batch_run(ral_batch* batch, void* stream, int32_t use_graph) {
    return guarded([&] {
        if (!batch) return set_error(kInvalidArgument, "null batch");
        cudaStream_t st = stream ? (cudaStream_t)stream : cudaStreamPerThread;
        return batch->b.run(st, use_graph != 0);
    });
}

int ral_batch_info(const ral_batch* batch, int32_t* num_programs, int64_t* total_rows, int64_t* work_items) {
    if (!batch) return set_error(kInvalidArgument, "null batch");
    if (num_programs) *num_programs = batch->b.programs();
    if (total_rows) *total_rows = batch->b.total_rows();
    if (work_items) *work_items = batch->b.total_items();
    return kSuccess;
}

int ral_batch_kernel_info(const ral_batch* batch, int32_t* registers, int32_t* grid, int32_t* blocks_per_sm) {
    if (!batch) return set_error(kInvalidArgument, "null batch");
    if (registers) *registers = batch->b.registers();
    if (grid) *grid = batch->b.grid();
    if (blocks_per_sm) *blocks_per_sm = batch->b.blocks_per_sm();
    return kSuccess;
}

int ral_batch_debug_source(const ral_batch* batch, int32_t compile, char* source_out, int64_t source_capacity,
                           char* log_out, int64_t log_capacity) {
    return guarded([&] {
        if (!batch) return set_error(kInvalidArgument, "null batch");
        std::string src, log;
        int rc = batch->b.debug_source(compile != 0, src, log);
        copy_out(std::string(jit_prelude()) + "\n" + src, source_out, source_capacity);
        copy_out(log, log_out, log_capacity);
        return rc;
    });
}

int ral_batch_destroy(ral_batch* batch) {
    delete batch;
    return kSuccess;
}

int ral_batch_tune_key(gdf_column* const* output_columns, int32_t num_outputs, gdf_column* const* input_columns,
                       int32_t num_inputs, const column_index_type* left_inputs, const column_index_type* right_inputs,
                       const column_index_type* outputs, int32_t num_operations,
                       const column_index_type* final_output_positions, const int32_t* operators,
                       const int32_t* unary_operators, const gdf_scalar* left_scalars, const gdf_scalar* right_scalars,
                       char* key_out, int64_t key_capacity) {
    return guarded([&] {
        ProgramArrays pa{left_inputs, right_inputs, outputs, num_operations, final_output_positions,
                         operators, unary_operators, left_scalars, right_scalars};
        Program p;
        if (int e = build_program(p, output_columns, num_outputs, input_columns, num_inputs, pa, false)) return e;
        copy_out(tune_key(p, 16 / max_width(p)), key_out, key_capacity);
        return (int)kSuccess;
    });
}

int ral_autotune_program(gdf_column* const* output_columns, int32_t num_outputs, gdf_column* const* input_columns,
                         int32_t num_inputs, const column_index_type* left_inputs,
                         const column_index_type* right_inputs, const column_index_type* outputs,
                         int32_t num_operations, const column_index_type* final_output_positions,
                         const int32_t* operators, const int32_t* unary_operators, const gdf_scalar* left_scalars,
                         const gdf_scalar* right_scalars, int32_t* best_slices, int32_t* best_unroll,
                         int32_t* best_soft_fp, double* best_ms) {
    return guarded([&] {
        ProgramArrays pa{left_inputs, right_inputs, outputs, num_operations, final_output_positions,
                         operators, unary_operators, left_scalars, right_scalars};
        Program p;
        if (int e = build_program(p, output_columns, num_outputs, input_columns, num_inputs, pa, false)) return e;
        const int G = 16 / max_width(p);
        // candidates: rows per item 32*G*J, slice loop unrolled U times; all compiled up front
        struct Cand { int J, U; bool S; };
        std::vector<Cand> cand;
        for (int S : {0, 1})
            for (int J : {2, 4, 8, 16})
                for (int U : {1, 2})
                    if (U <= J && (int64_t)32 * G * J <= 8192) cand.push_back({J, U, S != 0});
        std::vector<std::unique_ptr<ral_batch_s>> bs;
        for (auto& c : cand) {
            auto b = std::make_unique<ral_batch_s>();
            const int idx = b->b.add(output_columns, num_outputs, input_columns, num_inputs, pa);
            if (idx < 0) return -idx;
            b->b.force_shape(c.J, c.U, c.S);
            bs.push_back(std::move(b));
        }
        {   // compile every candidate's item and dispatcher at once, on the host thread pool
            std::vector<GeneratedKernel> tus;
            for (auto& c : cand) {
                Shape sh = tuned_shape(p, G);
                sh.J = c.J;
                sh.unroll = c.U;
                sh.soft = c.S;
                tus.push_back(generate_batch_item(p, sh));
                tus.push_back(generate_batch_dispatch({{tus.back().name, false}}, 0, batch_grab()));
            }
            std::vector<const std::vector<char>*> objs;
            if (int e = compile_items(tus, objs, nullptr)) return e;
        }
        cudaStream_t st = cudaStreamPerThread;
        for (auto& b : bs)
            if (int e = b->b.prepare(st)) return e;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        int bi = 0;
        double best = 1e30;
        for (size_t i = 0; i < bs.size(); i++) {
            int rc = bs[i]->b.run(st, true);
            cudaEventRecord(e0, st);
            for (int k = 0; k < 5 && !rc; k++) rc = bs[i]->b.run(st, true);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms / 5 < best) { best = ms / 5; bi = (int)i; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        record_tuned_shape(p, G, cand[bi].J, cand[bi].U, cand[bi].S, best);
        if (best_slices) *best_slices = cand[bi].J;
        if (best_unroll) *best_unroll = cand[bi].U;
        if (best_soft_fp) *best_soft_fp = cand[bi].S ? 1 : 0;
        if (best_ms) *best_ms = best;
        return check_cuda(cudaGetLastError(), "autotune");
    });
}

int64_t ral_kernel_launches(void) { return (int64_t)launch_count(); }

int ral_jit_stats(int64_t* compiles, int64_t* disk_hits, int64_t* memory_hits, double* compile_ms) {
    JitStats s = jit_stats();
    if (compiles) *compiles = s.compiles;
    if (disk_hits) *disk_hits = s.disk_hits;
    if (memory_hits) *memory_hits = s.memory_hits;
    if (compile_ms) *compile_ms = s.compile_ms_total;
    return 0;
}

int ral_server_create(int64_t budget_bytes, int32_t max_waves, int32_t max_wave_requests, int64_t wave_rows,
                      ral_server** server) {
    return guarded([&] {
        if (!server || budget_bytes <= 0 || wave_rows < 0) return set_error(kInvalidArgument, "bad argument");
        *server = new ral_server_s((size_t)budget_bytes, max_waves, max_wave_requests, wave_rows);
        return (int)kSuccess;
    });
}

int ral_server_add_table(ral_server* server, gdf_column* const* columns, int32_t num_columns, int32_t* table_id) {
    return guarded([&] {
        if (!server) return set_error(kInvalidArgument, "null server");
        int id = -1;
        int rc = server->s.add_table(columns, num_columns, &id);
        if (!rc && table_id) *table_id = id;
        return rc;
    });
}

int ral_server_add_query(ral_server* server, int32_t table_id, const char* filter_query_part,
                         const char* project_query_part, int32_t* query_id) {
    return guarded([&] {
        if (!server) return set_error(kInvalidArgument, "null server");
        int id = -1;
        int rc = server->s.add_query(table_id, filter_query_part, project_query_part, &id);
        if (!rc && query_id) *query_id = id;
        return rc;
    });
}

int ral_server_query_outputs(ral_server* server, int32_t query_id, gdf_dtype* dtypes, int32_t* has_valid,
                             int32_t capacity, int32_t* num_outputs) {
    return guarded([&] {
        if (!server) return set_error(kInvalidArgument, "null server");
        std::vector<gdf_dtype> d;
        std::vector<bool> v;
        if (int e = server->s.query_outputs(query_id, d, v)) return e;
        if ((int)d.size() > capacity) return set_error(kInvalidArgument, "capacity too small");
        for (size_t i = 0; i < d.size(); i++) {
            dtypes[i] = d[i];
            has_valid[i] = v[i] ? 1 : 0;
        }
        if (num_outputs) *num_outputs = (int32_t)d.size();
        return (int)kSuccess;
    });
}

int ral_server_debug_compile(ral_server* server, char* log_out, int64_t log_capacity) {
    return guarded([&] {
        if (!server) return set_error(kInvalidArgument, "null server");
        std::string log;
        int rc = server->s.debug_compile(log);
        copy_out(log, log_out, log_capacity);
        return rc;
    });
}

int ral_server_start(ral_server* server) {
    return guarded([&] {
        if (!server) return set_error(kInvalidArgument, "null server");
        return server->s.start();
    });
}

int ral_server_submit(ral_server* server, int32_t query_id, int32_t keep, int64_t* request_id) {
    return guarded([&] {
        if (!server) return set_error(kInvalidArgument, "null server");
        return server->s.submit(query_id, keep != 0, request_id);
    });
}

int ral_server_wait(ral_server* server, int64_t request_id, double timeout_s, int64_t* rows_out, double* latency_s) {
    return guarded([&] {
        if (!server) return set_error(kInvalidArgument, "null server");
        return server->s.wait(request_id, timeout_s, rows_out, latency_s);
    });
}

int ral_server_result(ral_server* server, int64_t request_id, gdf_column* out_columns, int32_t num_outputs) {
    return guarded([&] {
        if (!server || !out_columns) return set_error(kInvalidArgument, "null argument");
        return server->s.result(request_id, out_columns, num_outputs);
    });
}

int ral_server_copy_result(ral_server* server, int64_t request_id, gdf_column* const* out_columns,
                           int32_t num_outputs) {
    return guarded([&] {
        if (!server || !out_columns || num_outputs <= 0) return set_error(kInvalidArgument, "bad argument");
        std::vector<gdf_column> src(num_outputs);
        if (int e = server->s.result(request_id, src.data(), num_outputs)) return e;
        cudaStream_t st = cudaStreamPerThread;
        for (int o = 0; o < num_outputs; o++) {
            gdf_column* d = out_columns[o];
            if (!d) return set_error(kInvalidArgument, "null out column");
            if (d->dtype != src[o].dtype) return set_error(kInvalidArgument, "out column has the wrong dtype");
            if ((d->valid != nullptr) != (src[o].valid != nullptr))
                return set_error(kInvalidArgument, "out column mask presence differs from the query's");
            const size_t nb = (size_t)src[o].size * gdf_dtype_size(src[o].dtype);
            if (nb) cudaMemcpyAsync(d->data, src[o].data, nb, cudaMemcpyDeviceToDevice, st);
            if (src[o].valid && src[o].size)
                cudaMemcpyAsync(d->valid, src[o].valid, ((size_t)src[o].size + 7) / 8, cudaMemcpyDeviceToDevice, st);
            d->size = src[o].size;
            d->null_count = src[o].null_count;
        }
        return check_cuda(cudaStreamSynchronize(st), "copy of a served result");
    });
}

int ral_server_release(ral_server* server, int64_t request_id) {
    return guarded([&] {
        if (!server) return set_error(kInvalidArgument, "null server");
        return server->s.release(request_id);
    });
}

int ral_server_run_trace(ral_server* server, int32_t num_requests, const int32_t* queries, const double* arrival_s,
                         double* latency_s, int64_t* rows_out, double* makespan_s) {
    return guarded([&] {
        if (!server || num_requests < 0 || (num_requests > 0 && (!queries || !arrival_s)))
            return set_error(kInvalidArgument, "bad argument");
        return server->s.run_trace(num_requests, queries, arrival_s, latency_s, rows_out, makespan_s);
    });
}

int ral_server_stats(ral_server* server, int64_t* stats6) {
    if (!server || !stats6) return set_error(kInvalidArgument, "null argument");
    ServerStats st = server->s.stats();
    stats6[0] = st.submitted;
    stats6[1] = st.completed;
    stats6[2] = st.waves;
    stats6[3] = st.max_wave_requests;
    stats6[4] = (int64_t)st.peak_reserved;
    stats6[5] = (int64_t)(st.busy_s * 1e6);
    return kSuccess;
}

int ral_server_debug_stats(ral_server* server, int64_t* solo_requests, double* queue_s, double* run_s) {
    if (!server) return set_error(kInvalidArgument, "null argument");
    const ServerStats st = server->s.stats();
    if (solo_requests) *solo_requests = st.solo;
    if (queue_s) *queue_s = st.queue_s;
    if (run_s) *run_s = st.run_s;
    return kSuccess;
}

int ral_server_destroy(ral_server* server) {
    delete server;
    return kSuccess;
}

int ral_softfp_selftest(int64_t n, uint64_t seed, int64_t* mismatches, uint64_t* first_operands) {
    return guarded([&] {
        if (!mismatches || !first_operands || n < 0) return set_error(kInvalidArgument, "bad argument");
        std::vector<long long> c(16);
        std::vector<unsigned long long> f(32);
        int rc = softfp_selftest((long long)n, (unsigned long long)seed, c.data(), f.data());
        for (int i = 0; i < 16; i++) mismatches[i] = c[i];
        for (int i = 0; i < 32; i++) first_operands[i] = f[i];
        return rc;
    });
}

int ral_debug_lookback_timeout(int64_t n_rows, int32_t* status, int64_t* kept_after) {
    return guarded([&] {
        if (n_rows <= (int64_t)kCompactTileRows || n_rows > ((int64_t)64 << 20) || !status || !kept_after)
            return set_error(kInvalidArgument, "n_rows must be above one tile and at most 64M");
        cudaStream_t st = cudaStreamPerThread;
        const int64_t words = compact_scratch_words(n_rows);
        int8_t* stencil = nullptr;
        int32_t* idx = nullptr;
        unsigned long long* scratch = nullptr;
        auto cleanup = [&] {
            if (stencil) cudaFree(stencil);
            if (idx) cudaFree(idx);
            if (scratch) cudaFree(scratch);
        };
        if (check_cuda(cudaMalloc(&stencil, (size_t)n_rows), "cudaMalloc") ||
            check_cuda(cudaMalloc(&idx, (size_t)n_rows * 4), "cudaMalloc") ||
            check_cuda(cudaMalloc(&scratch, (size_t)words * 8), "cudaMalloc")) {
            cleanup();
            return (int)kCudaError;
        }
        cudaMemsetAsync(stencil, 1, (size_t)n_rows, st);
        // the ticket counter starts at 1: tile 0 is never taken, so tile 1's look-back waits on a
        // status word that nothing writes until its spin limit ends the wait
        cudaMemsetAsync(scratch, 0, (size_t)words * 8, st);
        const unsigned long long one = 1;
        cudaMemcpyAsync(scratch, &one, 8, cudaMemcpyHostToDevice, st);
        int rc = check_cuda(launch_compact_stencil(stencil, nullptr, n_rows, idx, scratch, st), "compaction");
        unsigned long long err = 0;
        if (!rc) cudaMemcpyAsync(&err, scratch + 1, 8, cudaMemcpyDeviceToHost, st);
        if (!rc) rc = check_cuda(cudaStreamSynchronize(st), "compaction with an unclaimed tile");
        *status = err ? (int32_t)kTimeout : (int32_t)kSuccess;
        // the context is still usable: the same compaction with every tile taken
        unsigned long long kept = 0;
        if (!rc) {
            cudaMemsetAsync(scratch, 0, (size_t)words * 8, st);
            rc = check_cuda(launch_compact_stencil(stencil, nullptr, n_rows, idx, scratch, st), "compaction");
            if (!rc) cudaMemcpyAsync(&kept, scratch + 2, 8, cudaMemcpyDeviceToHost, st);
            if (!rc) rc = check_cuda(cudaStreamSynchronize(st), "compaction");
        }
        *kept_after = (int64_t)kept;
        cleanup();
        return rc;
    });
}

}  // extern "C"
