// textscan.h — a table scan over delimited text in device memory fused with its LogicalFilter.
#pragma once

#include <cstdint>
#include <string>

#include "ral/gdf_compat.h"

namespace ral {

// Rows of data[0, n): lines (ending at term; the last may lack it) after the first skip_rows that
// are not blank once a '\r' before the terminator is dropped.
int text_scan_rows(const char* data, int64_t n, char term, int32_t skip_rows, int64_t* rows);

// The scan of the projected file columns, filtered by filter_q (null: every row), into outs
// (capacity = their size); see ral_text_scan_filter in ral_c.h.
int text_scan_filter(const char* data, int64_t n, char delim, char term, int32_t skip_rows, const int32_t* file_dtypes,
                     int32_t n_file, const int32_t* projections, int32_t n_proj, const char* filter_q,
                     gdf_column* const* outs, gdf_size_type* n_out);
// The same over text in host memory, copied in pieces of whole lines that are scanned while the
// next pieces are copied; see ral_text_scan_filter_host in ral_c.h.
int text_scan_filter_host(const char* text, int64_t n, char delim, char term, int32_t skip_rows,
                          const int32_t* file_dtypes, int32_t n_file, const int32_t* projections, int32_t n_proj,
                          const char* filter_q, gdf_column* const* outs, gdf_size_type* n_out);

// Generated source (and optionally an NVRTC-only compile) of the scan kernel; needs no GPU.
int text_scan_source(const int32_t* file_dtypes, int32_t n_file, const int32_t* projections, int32_t n_proj,
                     const char* filter_q, bool compile, std::string& source, std::string& log);

// Parquet (parquet_scan.cpp): the file's rows, leaf count and the dtype each leaf scans as
// (GDF_invalid where unsupported); the scan of the projected leaves filtered by filter_q.
int parquet_schema(const uint8_t* file, int64_t n, int64_t* rows, int32_t* n_columns, int32_t* dtypes, int32_t capacity);
int parquet_scan_filter(const uint8_t* file, int64_t n, const int32_t* projections, int32_t n_proj, const char* filter_q,
                        gdf_column* const* outs, gdf_size_type* n_out);

}  // namespace ral
