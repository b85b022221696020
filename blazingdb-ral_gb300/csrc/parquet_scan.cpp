// parquet_scan.cpp — a table scan over a Parquet file followed by its LogicalFilter.
//
// The reference scans a Parquet table in CalciteInterpreter.cpp:745-767 (BindableTableScan:
// `projects=[...]` picks the columns) through parquet_parser::parse
// (src/io/data_parser/ParquetParser.cpp:36-90, cudf's Parquet reader), and a LogicalFilter above
// it evaluates its condition over the scanned frame and compacts it (CalciteInterpreter.cpp:509).
// Here the footer and page headers are read on the host (parquet_meta.cpp), the projected columns'
// chunks are copied to the device in batches of pages, each batch decoded while the next is copied
// (a levels kernel for optional pages, a values kernel over 8192-row items of every page), and the
// fused filter kernel (filter.cpp) filters the columns -- or, without a filter, the decoded columns
// are the result.  Supported: flat schemas; INT32 (DATE), INT64 (TIMESTAMP_MILLIS), FLOAT, DOUBLE;
// required and optional columns; uncompressed v1 data pages with PLAIN values.  Anything else
// (compression, dictionary pages, other encodings or types) is refused with RAL_ERROR_UNSUPPORTED.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
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

// Pages go to the device in batches of about this many bytes (RAL_PARQUET_BATCH_BYTES overrides),
// each copied while the one before it is decoded.
int64_t batch_bytes() {
    const char* e = std::getenv("RAL_PARQUET_BATCH_BYTES");
    const long long v = e ? std::atoll(e) : 0;
    return v > 0 ? (int64_t)v : ((int64_t)24 << 20);
}

// The address kernels read file[0, n) at when it is page-locked (or mapped) host memory of this
// process, else null.  Both ends are checked: a registered range covers the whole buffer.
const uint8_t* device_view(const uint8_t* file, int64_t n) {
    if (std::getenv("RAL_PARQUET_STAGED")) return nullptr;  // always copy the chunks in
    cudaPointerAttributes a{}, b{};
    if (cudaPointerGetAttributes(&a, file) != cudaSuccess || cudaPointerGetAttributes(&b, file + n - 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer || !b.devicePointer) return nullptr;
    if ((const uint8_t*)b.devicePointer != (const uint8_t*)a.devicePointer + (n - 1)) return nullptr;
    return (const uint8_t*)a.devicePointer;
}

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
    std::vector<char> optional(n_proj, 0);
    for (int q = 0; q < n_proj; q++) {
        const int c = projections[q];
        if (c < 0 || c >= (int)meta.leaves.size()) return set_error(kInvalidArgument, "projection out of range");
        const pq::SchemaLeaf& l = meta.leaves[c];
        dtypes[q] = leaf_dtype(l);
        if (dtypes[q] == GDF_invalid)
            return set_error(kUnsupported, "column '" + l.name + "': only INT32 (DATE), INT64 (TIMESTAMP_MILLIS), FLOAT "
                                           "and DOUBLE columns are scanned");
        if (l.repetition == 2) return set_error(kUnsupported, "column '" + l.name + "' is repeated");
        optional[q] = l.repetition == 1;
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
    std::vector<int64_t> page_file;  // each page's data offset in the file
    struct Range {
        int64_t file_off, bytes, dev_off;
    };
    std::vector<Range> ranges;
    std::vector<int32_t> page_range;
    int64_t packed = 0, items = 0;
    int64_t row0 = 0;
    for (const pq::RowGroupMeta& g : meta.row_groups) {
        for (int q = 0; q < n_proj; q++) {
            const pq::ColumnChunkMeta& cc = g.columns[projections[q]];
            const pq::SchemaLeaf& l = meta.leaves[projections[q]];
            const int w = gdf_dtype_size(dtypes[q]);
            if (cc.codec != 0) return set_error(kUnsupported, "column '" + l.name + "': compressed column chunks are not supported");
            if (cc.dictionary_page_offset >= 0)
                return set_error(kUnsupported, "column '" + l.name + "': dictionary-encoded pages are not supported");
            int64_t at = cc.data_page_offset, seen = 0;
            const size_t first_page = pages.size();
            while (seen < cc.num_values) {
                pq::PageHeader ph;
                const std::string err = pq::read_page_header(file, n, at, ph);
                if (!err.empty()) return set_error(kUnsupported, err);
                if (ph.type != 0 || ph.encoding != 0 || (optional[q] && ph.def_encoding != 3) ||
                    ph.compressed_size != ph.uncompressed_size)
                    return set_error(kUnsupported, "column '" + l.name + "': only uncompressed v1 data pages of PLAIN "
                                                   "values (RLE definition levels) are supported");
                const int64_t data = at + ph.header_bytes;
                if (ph.num_values < 0 || ph.compressed_size < 0 || data + ph.compressed_size > n)
                    return set_error(kUnsupported, "column '" + l.name + "': a page runs past the end of the file");
                ParquetPage p{};
                p.row_start = row0 + seen;
                p.rows = ph.num_values;
                p.data_bytes = ph.compressed_size;
                p.column = q;
                p.optional = optional[q];
                if (p.rows > 0) {
                    // the levels' length is read here; the values of a required page are checked here
                    // and an optional page's against its levels on the device
                    bool ok;
                    if (p.optional) {
                        ok = p.data_bytes >= 4;
                        if (ok) {
                            const uint8_t* d = file + data;
                            const int64_t lev = (int64_t)((uint32_t)d[0] | (uint32_t)d[1] << 8 | (uint32_t)d[2] << 16 |
                                                          (uint32_t)d[3] << 24);
                            ok = 4 + lev <= p.data_bytes;
                            p.levels = (int32_t)lev;
                        }
                    } else {
                        ok = (int64_t)p.data_bytes / w >= p.rows;
                    }
                    if (!ok) return set_error(kUnsupported, "column '" + l.name + "': a data page whose levels or values run past its data");
                    p.item0 = (int32_t)items;
                    items += (p.rows + kParquetItemRows - 1) / kParquetItemRows;
                    pages.push_back(p);
                    page_file.push_back(data);
                    page_range.push_back((int32_t)ranges.size());
                }
                seen += ph.num_values;
                at = data + ph.compressed_size;
            }
            if (seen != g.num_rows) return set_error(kUnsupported, "column '" + l.name + "': page values differ from the row group's rows");
            const Range r{cc.data_page_offset, at - cc.data_page_offset, packed};
            for (size_t k = first_page; k < pages.size(); k++) pages[k].data = r.dev_off + (page_file[k] - r.file_off);
            ranges.push_back(r);
            packed += (r.bytes + 15) & ~15ll;
        }
        row0 += g.num_rows;
    }
    if (row0 != rows) return set_error(kUnsupported, "row groups do not add up to the file's rows");
    if (pages.size() > (size_t)INT32_MAX || items > (int64_t)INT32_MAX) return set_error(kUnsupported, "too many pages");

    cudaStream_t st = cudaStreamPerThread;
    keep_pool_memory();
    CopyLane* lane = nullptr;
    if (int e = copy_lane(lane)) return e;
    DevBuf dfile(st), dpages(st), dstatus(st), ditems(st);
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
        // a required column's rows are all present; an optional column's bits are set by the levels
        const size_t mbytes = gdf_valid_allocation_size(std::max<int64_t>(rows, 1));
        cudaMemsetAsync(frame[q].valid, 0, mbytes, st);
        if (!optional[q] && rows > 0) {
            if (rows >= 8) cudaMemsetAsync(frame[q].valid, 0xff, (size_t)(rows / 8), st);
            if (rows % 8) cudaMemsetAsync((char*)frame[q].valid + rows / 8, (1 << (rows % 8)) - 1, 1, st);
        }
    }
    // A page-locked file is read by the kernels where it lies (over the host link, no staging copy);
    // any other host memory is copied in.
    const uint8_t* direct = device_view(file, n);
    if (direct)
        for (size_t k = 0; k < pages.size(); k++) pages[k].data = page_file[k];
    else if (int e = dfile.alloc((size_t)packed))
        return e;
    if (int e = dpages.alloc(pages.size() * sizeof(ParquetPage))) return e;
    if (!pages.empty() &&
        check_cuda(cudaMemcpyAsync(dpages.p, pages.data(), pages.size() * sizeof(ParquetPage), cudaMemcpyHostToDevice, st),
                   "cudaMemcpyAsync"))
        return kCudaError;
    if (int e = dstatus.alloc((size_t)(1 + n_proj) * 8)) return e;
    cudaMemsetAsync(dstatus.p, 0, (size_t)(1 + n_proj) * 8, st);
    if (int e = ditems.alloc((size_t)items * 4)) return e;
    cudaMemsetAsync(ditems.p, 0, (size_t)items * 4, st);
    ParquetDecodeParams dp{};
    dp.file = direct ? direct : (const uint8_t*)dfile.p;
    dp.pages = (const ParquetPage*)dpages.p;
    dp.status = (unsigned long long*)dstatus.p;
    dp.item_base = (uint32_t*)ditems.p;
    for (int q = 0; q < n_proj; q++) {
        dp.out[q].data = frame[q].data;
        dp.out[q].valid = (uint32_t*)frame[q].valid;
        dp.out[q].width = gdf_dtype_size(dtypes[q]);
    }
    bool any_optional = false;
    for (const char o : optional) any_optional |= o != 0;
    if (direct && !pages.empty()) {
        dp.page_lo = 0;
        dp.page_hi = (int32_t)pages.size();
        dp.item_lo = 0;
        dp.item_hi = (int32_t)items;
        if (any_optional && check_cuda(launch_parquet_levels(dp, st), "Parquet definition levels")) return kCudaError;
        if (int e = check_cuda(launch_parquet_values(dp, st), "Parquet page values")) return e;
    }
    // Otherwise the pages go in batches of about kBatchBytes: a batch's bytes are copied on the copy
    // lane's stream while the batch before it is decoded on this one.
    if (int e = check_cuda(cudaEventRecord(lane->ready, st), "cudaEventRecord")) return e;
    if (int e = check_cuda(cudaStreamWaitEvent(lane->s, lane->ready, 0), "cudaStreamWaitEvent")) return e;
    LaneJoin join{lane, st};  // before the buffers are freed, this stream waits for every copy
    const int64_t kBatchBytes = batch_bytes();
    size_t batch = 0;
    for (size_t p0 = direct ? pages.size() : 0; p0 < pages.size(); batch++) {
        size_t p1 = p0;
        int64_t bytes = 0;
        bool batch_optional = false;
        while (p1 < pages.size() && (p1 == p0 || bytes < kBatchBytes)) {
            bytes += pages[p1].data_bytes;
            batch_optional |= pages[p1].optional != 0;
            p1++;
        }
        // one copy per run of pages from the same column chunk (their data and headers between)
        for (size_t a = p0; a < p1;) {
            size_t b = a;
            while (b + 1 < p1 && page_range[b + 1] == page_range[a]) b++;
            const int64_t f0 = page_file[a], f1 = page_file[b] + pages[b].data_bytes;
            if (f1 > f0 && check_cuda(cudaMemcpyAsync((char*)dfile.p + pages[a].data, file + f0, (size_t)(f1 - f0),
                                                      cudaMemcpyHostToDevice, lane->s),
                                      "cudaMemcpyAsync"))
                return kCudaError;
            a = b + 1;
        }
        cudaEvent_t copied = nullptr;
        if (int e = lane_event(*lane, batch, &copied)) return e;
        if (int e = check_cuda(cudaEventRecord(copied, lane->s), "cudaEventRecord")) return e;
        if (int e = check_cuda(cudaStreamWaitEvent(st, copied, 0), "cudaStreamWaitEvent")) return e;
        dp.page_lo = (int32_t)p0;
        dp.page_hi = (int32_t)p1;
        dp.item_lo = pages[p0].item0;
        dp.item_hi = p1 < pages.size() ? pages[p1].item0 : (int32_t)items;
        if (batch_optional && check_cuda(launch_parquet_levels(dp, st), "Parquet definition levels")) return kCudaError;
        if (int e = check_cuda(launch_parquet_values(dp, st), "Parquet page values")) return e;
        p0 = p1;
    }
    std::vector<unsigned long long> status(1 + n_proj, 0);
    if (int e = check_cuda(cudaMemcpyAsync(status.data(), dstatus.p, status.size() * 8, cudaMemcpyDeviceToHost, st),
                           "cudaMemcpyAsync"))
        return e;
    if (int e = check_cuda(cudaStreamSynchronize(st), "Parquet page decode")) return e;
    if (status[0]) return set_error(kUnsupported, std::to_string(status[0]) + " data pages whose levels or values run past their data");
    for (int q = 0; q < n_proj; q++)
        frame[q].null_count = optional[q] ? (gdf_size_type)(rows - (int64_t)status[1 + q]) : 0;
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
