// parquet_scan.cpp — a table scan over a Parquet file followed by its LogicalFilter.
//
// The reference scans a Parquet table in CalciteInterpreter.cpp:745-767 (BindableTableScan:
// `projects=[...]` picks the columns) through parquet_parser::parse
// (src/io/data_parser/ParquetParser.cpp:36-90, cudf's Parquet reader), and a LogicalFilter above
// it evaluates its condition over the scanned frame and compacts it (CalciteInterpreter.cpp:509).
// Here the footer and page headers are read on the host (parquet_meta.cpp), the projected columns'
// chunks are copied to the device (one copy each), one kernel decodes every data page into columns, and
// the fused filter kernel (filter.cpp) filters them -- or, without a filter, the decoded columns are
// the result.  Supported: flat schemas; INT32 (DATE), INT64 (TIMESTAMP_MILLIS), FLOAT, DOUBLE;
// required and optional columns; uncompressed v1 data pages with PLAIN values.  Anything else
// (compression, dictionary pages, other encodings or types) is refused with RAL_ERROR_UNSUPPORTED.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"
#include "filter.h"
#include "kernels.h"
#include "parquet_meta.h"
#include "ral/ral_c.h"

namespace ral {

namespace {

struct DevBuf {
    void* p = nullptr;
    cudaStream_t st = nullptr;
    explicit DevBuf(cudaStream_t s) : st(s) {}
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() {
        if (p) cudaFreeAsync(p, st);
    }
    int alloc(size_t bytes) { return check_cuda(cudaMallocAsync(&p, std::max<size_t>(bytes, 16), st), "cudaMallocAsync"); }
};

// The gdf dtype a supported leaf scans as, or GDF_invalid.
gdf_dtype leaf_dtype(const pq::SchemaLeaf& l) {
    switch (l.type) {
    case 1: return l.converted_type == 6 ? GDF_DATE32 : (l.converted_type == -1 ? GDF_INT32 : GDF_invalid);
    case 2: return l.converted_type == 9 ? GDF_DATE64 : (l.converted_type == -1 ? GDF_INT64 : GDF_invalid);
    case 4: return GDF_FLOAT32;
    case 5: return GDF_FLOAT64;
    default: return GDF_invalid;
    }
}

int read_meta(const uint8_t* file, int64_t n, pq::FileMeta& meta) {
    if (!file || n <= 0) return set_error(kInvalidArgument, "bad argument");
    const std::string err = pq::read_file_meta(file, n, meta);
    if (!err.empty()) return set_error(kUnsupported, err);
    return kSuccess;
}

}  // namespace

int parquet_schema(const uint8_t* file, int64_t n, int64_t* rows, int32_t* n_columns, int32_t* dtypes, int32_t capacity) {
    pq::FileMeta meta;
    if (int e = read_meta(file, n, meta)) return e;
    if (rows) *rows = meta.num_rows;
    if (n_columns) *n_columns = (int32_t)meta.leaves.size();
    if (dtypes)
        for (int32_t k = 0; k < capacity && k < (int32_t)meta.leaves.size(); k++) dtypes[k] = (int32_t)leaf_dtype(meta.leaves[k]);
    return kSuccess;
}

int parquet_scan_filter(const uint8_t* file, int64_t n, const int32_t* projections, int32_t n_proj, const char* filter_q,
                        gdf_column* const* outs, gdf_size_type* n_out) {
    if (!projections || n_proj <= 0 || !outs || !n_out) return set_error(kInvalidArgument, "bad argument");
    if (n_proj > kParquetMaxColumns) return set_error(kUnsupported, "more than 64 projected columns");
    pq::FileMeta meta;
    if (int e = read_meta(file, n, meta)) return e;
    const int64_t rows = meta.num_rows;
    if (rows > (int64_t)INT32_MAX) return set_error(kUnsupported, "more rows than a gdf_size_type holds");
    std::vector<gdf_dtype> dtypes(n_proj);
    for (int q = 0; q < n_proj; q++) {
        const int c = projections[q];
        if (c < 0 || c >= (int)meta.leaves.size()) return set_error(kInvalidArgument, "projection out of range");
        const pq::SchemaLeaf& l = meta.leaves[c];
        dtypes[q] = leaf_dtype(l);
        if (dtypes[q] == GDF_invalid)
            return set_error(kUnsupported, "column '" + l.name + "': only INT32 (DATE), INT64 (TIMESTAMP_MILLIS), FLOAT "
                                           "and DOUBLE columns are scanned");
        if (l.repetition == 2) return set_error(kUnsupported, "column '" + l.name + "' is repeated");
        if (!outs[q] || outs[q]->dtype != dtypes[q])
            return set_error(kInvalidArgument, "out column " + std::to_string(q) + " is missing or has the wrong dtype");
        if (!outs[q]->valid || ((uintptr_t)outs[q]->valid & 3))
            return set_error(kInvalidArgument, "out columns need a 4-byte aligned mask");
        if (outs[q]->size < rows)
            return set_error(kInvalidArgument, "out columns must hold every row of the file (" + std::to_string(rows) + ")");
    }
    // the data pages of the projected columns; only their column chunks travel to the device, packed
    // one after another (a page's `data` is its offset in that packed copy)
    std::vector<ParquetPage> pages;
    struct Range {
        int64_t file_off, bytes, dev_off;
    };
    std::vector<Range> ranges;
    int64_t packed = 0;
    int64_t row0 = 0;
    for (const pq::RowGroupMeta& g : meta.row_groups) {
        for (int q = 0; q < n_proj; q++) {
            const pq::ColumnChunkMeta& cc = g.columns[projections[q]];
            const pq::SchemaLeaf& l = meta.leaves[projections[q]];
            if (cc.codec != 0) return set_error(kUnsupported, "column '" + l.name + "': compressed column chunks are not supported");
            if (cc.dictionary_page_offset >= 0)
                return set_error(kUnsupported, "column '" + l.name + "': dictionary-encoded pages are not supported");
            int64_t at = cc.data_page_offset, seen = 0;
            const size_t first_page = pages.size();
            while (seen < cc.num_values) {
                pq::PageHeader ph;
                const std::string err = pq::read_page_header(file, n, at, ph);
                if (!err.empty()) return set_error(kUnsupported, err);
                if (ph.type != 0 || ph.encoding != 0 || (l.repetition == 1 && ph.def_encoding != 3) ||
                    ph.compressed_size != ph.uncompressed_size)
                    return set_error(kUnsupported, "column '" + l.name + "': only uncompressed v1 data pages of PLAIN "
                                                   "values (RLE definition levels) are supported");
                const int64_t data = at + ph.header_bytes;
                if (ph.num_values < 0 || ph.compressed_size < 0 || data + ph.compressed_size > n)
                    return set_error(kUnsupported, "column '" + l.name + "': a page runs past the end of the file");
                ParquetPage p{};
                p.row_start = row0 + seen;
                p.data = data;
                p.rows = ph.num_values;
                p.data_bytes = ph.compressed_size;
                p.column = q;
                p.optional = l.repetition == 1 ? 1 : 0;
                if (p.rows > 0) pages.push_back(p);
                seen += ph.num_values;
                at = data + ph.compressed_size;
            }
            if (seen != g.num_rows) return set_error(kUnsupported, "column '" + l.name + "': page values differ from the row group's rows");
            const Range r{cc.data_page_offset, at - cc.data_page_offset, packed};
            for (size_t k = first_page; k < pages.size(); k++) pages[k].data = r.dev_off + (pages[k].data - r.file_off);
            ranges.push_back(r);
            packed += (r.bytes + 15) & ~15ll;
        }
        row0 += g.num_rows;
    }
    if (row0 != rows) return set_error(kUnsupported, "row groups do not add up to the file's rows");
    if (pages.size() > (size_t)INT32_MAX) return set_error(kUnsupported, "too many pages");

    cudaStream_t st = cudaStreamPerThread;
    DevBuf dfile(st), dpages(st), dstatus(st);
    // decoded columns: the outputs themselves without a filter, a frame of temporaries with one
    std::vector<std::unique_ptr<DevBuf>> owned;
    std::vector<gdf_column> frame(n_proj);
    std::vector<gdf_column*> pframe(n_proj);
    for (int q = 0; q < n_proj; q++) {
        frame[q] = gdf_column{};
        frame[q].dtype = dtypes[q];
        frame[q].size = (gdf_size_type)rows;
        if (filter_q) {
            owned.emplace_back(new DevBuf(st));
            if (int e = owned.back()->alloc((size_t)rows * gdf_dtype_size(dtypes[q]) + gdf_valid_allocation_size(rows)))
                return e;
            frame[q].data = owned.back()->p;
            frame[q].valid = (gdf_valid_type*)((char*)owned.back()->p + (size_t)rows * gdf_dtype_size(dtypes[q]));
            // a multiple of 16 bytes keeps the mask 4-byte aligned
            if (((uintptr_t)frame[q].valid) & 3) return set_error(kInvalidArgument, "internal: unaligned mask");
        } else {
            frame[q].data = outs[q]->data;
            frame[q].valid = outs[q]->valid;
        }
        pframe[q] = &frame[q];
        cudaMemsetAsync(frame[q].valid, 0, gdf_valid_allocation_size(std::max<int64_t>(rows, 1)), st);
    }
    if (int e = dfile.alloc((size_t)packed)) return e;
    for (const Range& r : ranges)
        if (r.bytes > 0 && check_cuda(cudaMemcpyAsync((char*)dfile.p + r.dev_off, file + r.file_off, (size_t)r.bytes,
                                                      cudaMemcpyHostToDevice, st),
                                      "cudaMemcpyAsync"))
            return kCudaError;
    if (int e = dpages.alloc(pages.size() * sizeof(ParquetPage))) return e;
    if (!pages.empty() &&
        check_cuda(cudaMemcpyAsync(dpages.p, pages.data(), pages.size() * sizeof(ParquetPage), cudaMemcpyHostToDevice, st),
                   "cudaMemcpyAsync"))
        return kCudaError;
    if (int e = dstatus.alloc((size_t)(1 + n_proj) * 8)) return e;
    cudaMemsetAsync(dstatus.p, 0, (size_t)(1 + n_proj) * 8, st);
    ParquetDecodeParams dp{};
    dp.file = (const uint8_t*)dfile.p;
    dp.pages = (const ParquetPage*)dpages.p;
    dp.status = (unsigned long long*)dstatus.p;
    dp.num_pages = (int32_t)pages.size();
    dp.num_columns = n_proj;
    for (int q = 0; q < n_proj; q++) {
        dp.out[q].data = frame[q].data;
        dp.out[q].valid = (uint32_t*)frame[q].valid;
        dp.out[q].width = gdf_dtype_size(dtypes[q]);
    }
    if (int e = check_cuda(launch_parquet_decode(dp, st), "Parquet page decode")) return e;
    std::vector<unsigned long long> status(1 + n_proj, 0);
    if (int e = check_cuda(cudaMemcpyAsync(status.data(), dstatus.p, status.size() * 8, cudaMemcpyDeviceToHost, st),
                           "cudaMemcpyAsync"))
        return e;
    if (int e = check_cuda(cudaStreamSynchronize(st), "Parquet page decode")) return e;
    if (status[0]) return set_error(kUnsupported, std::to_string(status[0]) + " data pages whose levels or values run past their data");
    for (int q = 0; q < n_proj; q++) frame[q].null_count = (gdf_size_type)(rows - (int64_t)status[1 + q]);
    if (!filter_q) {
        for (int q = 0; q < n_proj; q++) {
            outs[q]->size = (gdf_size_type)rows;
            outs[q]->null_count = frame[q].null_count;
        }
        *n_out = (gdf_size_type)rows;
        return kSuccess;
    }
    FilterOptions opt;
    opt.stream = st;
    return process_filter(pframe.data(), n_proj, filter_q, outs, n_out, opt);
}

}  // namespace ral
