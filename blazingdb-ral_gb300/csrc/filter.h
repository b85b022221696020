// filter.h — LogicalFilter (process_filter) and the fused filter + project.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "codegen.h"
#include "program.h"
#include "ral/gdf_compat.h"

namespace ral {

struct FilterOptions {
    cudaStream_t stream = nullptr;
    bool sync = true;
    // 0: fused single kernel (default), 1: stencil -> compaction -> gather
    // (the reference's three steps, kept as a cross-check); RAL_FILTER_MODE overrides
    int mode = -1;
};

int process_filter(gdf_column* const* frame, int num_columns, const char* query_part, gdf_column* const* out_columns,
                   gdf_size_type* num_rows_out, const FilterOptions& opt);

// Generated source (and optionally an NVRTC-only compile) of the fused filter kernel
// for a frame described by dtype and mask presence; needs no GPU.
int debug_filter_source(gdf_column* const* frame, int num_columns, const char* filter_query_part,
                        const char* project_query_part, bool compile, std::string& source, std::string& log);

int filter_project(gdf_column* const* frame, int num_columns, const char* filter_query_part,
                   const char* project_query_part, gdf_column* const* out_columns, int num_out_columns,
                   gdf_size_type* num_rows_out, const FilterOptions& opt);

// process_filter (project_q null) or filter_project over columns in host memory, streamed through
// the GPU in chunks of chunk_rows (0: 4Mi) on three streams; outputs in host memory.
int filter_host(gdf_column* const* frame, int ncols, const char* filter_q, const char* project_q,
                gdf_column* const* outs, int n_outs, gdf_size_type* n_out, int64_t chunk_rows);

// The standalone fused filter + project kernel over a whole frame, for a caller that launches it
// itself (the served loop runs large requests this way): prepared (compiled) for a frame and the
// outputs' dtypes and mask presence; enqueue_standalone_filter zeroes the scratch and the output
// masks, launches, and copies the header (error word, kept count, valid counts) to host_header.
int prepare_standalone_filter(gdf_column* const* frame, int ncols, const char* filter_q, const char* project_q,
                              gdf_column* const* outs, int n_outs, const void** handle);
int64_t standalone_scratch_words(const void* handle, int64_t n);
int enqueue_standalone_filter(const void* handle, gdf_column* const* frame, gdf_column* const* outs, void* scratch,
                              unsigned long long* host_header, cudaStream_t st);

// Launches of fused filter kernels in grid mode (a cooperative launch with one grid barrier in
// place of the look-back) since the library was loaded.
int64_t filter_grid_launches();

// A LogicalProject over a LogicalFilter, planned for a frame: the fused filter's spec and the
// dtype / mask presence of every output (evaluated outputs carry a mask; a pass-through output
// carries one exactly when its frame column does).  Holds the programs the spec points to.
struct FilterPlan {
    FilterSpec spec;
    Program pred, proj;
    bool have_pred = false, have_proj = false;
    std::vector<gdf_dtype> out_dtypes;
    std::vector<bool> out_valid;
};
int plan_filter_project(gdf_column* const* frame, int ncols, const char* filter_query_part,
                        const char* project_query_part, std::unique_ptr<FilterPlan>& plan);

// Parameter slots of a fused filter launch (kernel or batch item) of the plan.
void filter_fill_slots(const FilterPlan& plan, const GeneratedKernel& gk, gdf_column* const* frame, int64_t n_rows,
                       void* const* out_data, void* const* out_valid, void* scratch, std::vector<uint64_t>& slots);

}  // namespace ral
