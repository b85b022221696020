// filter.h — LogicalFilter (process_filter) and the fused filter + project.
#pragma once

#include <cuda_runtime.h>

#include <string>

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

}  // namespace ral
