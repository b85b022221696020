// parquet_scan.cpp — a table scan over a Parquet file followed by its LogicalFilter.
//
// The reference scans a Parquet table in CalciteInterpreter.cpp:745-767 (BindableTableScan:
// `projects=[...]` picks the columns) through parquet_parser::parse
// (src/io/data_parser/ParquetParser.cpp:36-90, cudf's Parquet reader), and a LogicalFilter above
// it evaluates its condition over the scanned frame and compacts it (CalciteInterpreter.cpp:509).
// Here the footer and page headers are read on the host (parquet_meta.cpp) and the pages are
// decoded on the device: a page-locked file is read in place over the host link, other host memory
// is copied in, column chunk by column chunk, in batches decoded while the next batch is copied.
// Snappy-compressed pages are decompressed first (one warp per page), then a levels kernel decodes
// optional pages' definition levels, a dictionary kernel the indices of dictionary-encoded pages,
// and a values kernel every page's values in 8192-row items; the fused filter kernel (filter.cpp)
// filters the columns -- or, without a filter, the decoded columns are the result.  Supported: flat
// schemas; INT32 (DATE), INT64 (TIMESTAMP_MILLIS), FLOAT, DOUBLE; required and optional columns;
// v1 and v2 data pages of PLAIN values or dictionary indices (PLAIN_DICTIONARY / RLE_DICTIONARY);
// uncompressed or Snappy-compressed chunks.  Anything else (other codecs, encodings or types,
// nested schemas) is refused with RAL_ERROR_UNSUPPORTED.
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

// Where a page's bytes are read: in the file (chunk `chunk`, at file offset file_off), or in the
// unpack buffer at `unpack` (a Snappy page, decompressed there).
struct PageWhere {
    int64_t file_off = 0;
    int64_t unpack = -1;
    int32_t chunk = 0;
};
// A Snappy page body: src_bytes compressed bytes at file offset src_off (after `prefix` raw bytes,
// a v2 page's levels), decompressed to dst_bytes at dst_off of the unpack buffer after the prefix.
struct Unpack {
    int64_t src_off, src_bytes, dst_off, dst_bytes;
    int32_t prefix, chunk;
};
// A projected column chunk: its bytes in the file, its place in the staging copy, its pages and
// Snappy jobs.
struct Chunk {
    int64_t file_off = 0, bytes = 0, dev_off = 0;
    int32_t page_begin = 0, page_end = 0, unpack_begin = 0, unpack_end = 0;
};
struct ChunkPlan {
    std::vector<ParquetPage> pages;
    std::vector<PageWhere> where, dict_where;  // per page: its data, its dictionary
    std::vector<Chunk> chunks;
    std::vector<Unpack> unpacks;
    int64_t packed = 0, unpack_bytes = 0, items = 0, n_idx = 0;
};

// Reads every page header of the projected leaves' column chunks (dictionary pages, v1 and v2 data
// pages; index pages are passed over) and checks what can be checked before any device work.
int plan_chunks(const uint8_t* file, int64_t n, const pq::FileMeta& meta, const int32_t* projections, int n_proj,
                const std::vector<gdf_dtype>& dtypes, const std::vector<char>& optional, ChunkPlan& plan) {
    int64_t row0 = 0;
    for (const pq::RowGroupMeta& g : meta.row_groups) {
        for (int q = 0; q < n_proj; q++) {
            const pq::ColumnChunkMeta& cc = g.columns[projections[q]];
            const pq::SchemaLeaf& l = meta.leaves[projections[q]];
            const std::string col = "column '" + l.name + "': ";
            const int w = gdf_dtype_size(dtypes[q]);
            if (cc.codec != 0 && cc.codec != 1)
                return set_error(kUnsupported, col + "only uncompressed and Snappy-compressed column chunks are supported");
            const bool snappy = cc.codec == 1;
            // a dictionary page offset below 4 (inside the leading magic) means "none": some writers store 0
            const int64_t start = cc.dictionary_page_offset >= 4 ? std::min(cc.dictionary_page_offset, cc.data_page_offset)
                                                                 : cc.data_page_offset;
            Chunk ch;
            ch.file_off = start;
            ch.dev_off = plan.packed;
            ch.page_begin = (int32_t)plan.pages.size();
            ch.unpack_begin = (int32_t)plan.unpacks.size();
            const int32_t ci = (int32_t)plan.chunks.size();
            PageWhere dict_at;
            int32_t dict_count = 0;
            bool have_dict = false;
            int64_t at = start, seen = 0;
            while (seen < cc.num_values) {
                pq::PageHeader ph;
                const std::string err = pq::read_page_header(file, n, at, ph);
                if (!err.empty()) return set_error(kUnsupported, col + err);
                const int64_t data = at + ph.header_bytes;
                if (ph.num_values < 0 || ph.compressed_size < 0 || ph.uncompressed_size < 0 || data + ph.compressed_size > n)
                    return set_error(kUnsupported, col + "a page runs past the end of the file");
                at = data + ph.compressed_size;
                if (ph.type != 0 && ph.type != 2 && ph.type != 3) continue;  // index pages carry no values
                if (!snappy && ph.compressed_size != ph.uncompressed_size)
                    return set_error(kUnsupported, col + "a page of an uncompressed chunk whose sizes differ");
                // a Snappy page is decompressed into the unpack buffer: all of a v1 or dictionary
                // page, a v2 page's values after its raw levels (unless it says they are stored raw)
                const bool v2 = ph.type == 3;
                const int32_t raw = v2 ? ph.def_bytes + ph.rep_bytes : 0;
                if (v2 && (ph.def_bytes < 0 || ph.rep_bytes < 0 || raw > ph.compressed_size || raw > ph.uncompressed_size))
                    return set_error(kUnsupported, col + "a v2 page whose levels run past its data");
                PageWhere pw;
                pw.file_off = data;
                pw.chunk = ci;
                const bool unpack = snappy && (!v2 || ph.v2_compressed);
                if (unpack) {
                    pw.unpack = plan.unpack_bytes;
                    plan.unpacks.push_back({data + raw, (int64_t)ph.compressed_size - raw, plan.unpack_bytes,
                                            (int64_t)ph.uncompressed_size - raw, raw, ci});
                    // at least 16 bytes: the kernels' aligned reads near a page's start stay inside
                    plan.unpack_bytes += std::max<int64_t>(16, ((int64_t)ph.uncompressed_size + 15) & ~15ll);
                } else if (snappy && ph.compressed_size != ph.uncompressed_size) {
                    return set_error(kUnsupported, col + "a page stored raw whose sizes differ");
                }
                const int32_t bytes = ph.uncompressed_size;
                if (ph.type == 2) {
                    if (ph.encoding != 0 && ph.encoding != 2)
                        return set_error(kUnsupported, col + "a dictionary page not of PLAIN values");
                    if ((int64_t)ph.num_values * w > bytes) return set_error(kUnsupported, col + "a dictionary page shorter than its entries");
                    dict_at = pw;
                    dict_count = ph.num_values;
                    have_dict = true;
                    continue;
                }
                const bool dict_enc = ph.encoding == 2 || ph.encoding == 8;
                if (ph.encoding != 0 && !dict_enc)
                    return set_error(kUnsupported, col + "page encoding " + std::to_string(ph.encoding) +
                                                   " (only PLAIN values and dictionary indices are supported)");
                if (dict_enc && (!have_dict || dict_count <= 0))
                    return set_error(kUnsupported, col + "a dictionary-encoded page without a dictionary");
                if (v2 && ph.rep_bytes != 0) return set_error(kUnsupported, col + "repetition levels in a flat schema");
                ParquetPage p{};
                p.row_start = row0 + seen;
                p.rows = ph.num_values;
                p.data_bytes = bytes;
                p.column = q;
                p.optional = optional[q];
                seen += ph.num_values;
                if (p.rows <= 0) continue;
                if (v2) {
                    p.levels = p.optional ? ph.def_bytes : 0;
                    p.values_off = ph.def_bytes;
                } else if (p.optional) {
                    if (ph.def_encoding != 3) return set_error(kUnsupported, col + "definition levels not in the RLE hybrid");
                    // the level runs' length leads a v1 page: read here, or for a Snappy page from
                    // its decompressed bytes on the device
                    p.lev_off = 4;
                    if (unpack) {
                        p.levels = -1;
                    } else {
                        if (bytes < 4) return set_error(kUnsupported, col + "a data page shorter than its levels");
                        const uint8_t* d = file + data;
                        p.levels = (int32_t)((uint32_t)d[0] | (uint32_t)d[1] << 8 | (uint32_t)d[2] << 16 | (uint32_t)d[3] << 24);
                        if (p.levels < 0 || 4 + (int64_t)p.levels > bytes)
                            return set_error(kUnsupported, col + "a data page whose levels run past its data");
                        p.values_off = 4 + p.levels;
                    }
                }
                if (p.values_off > bytes) return set_error(kUnsupported, col + "a data page whose levels run past its data");
                if (!dict_enc && !p.optional && (int64_t)(bytes - p.values_off) / w < p.rows)
                    return set_error(kUnsupported, col + "a data page whose values run past its data");
                if (dict_enc) {
                    p.dict_count = dict_count;
                    p.idx0 = (int32_t)plan.n_idx;
                    plan.n_idx += p.rows;
                }
                p.item0 = (int32_t)plan.items;
                plan.items += (p.rows + kParquetItemRows - 1) / kParquetItemRows;
                plan.pages.push_back(p);
                plan.where.push_back(pw);
                plan.dict_where.push_back(dict_enc ? dict_at : PageWhere{});
            }
            if (seen != g.num_rows) return set_error(kUnsupported, col + "page values differ from the row group's rows");
            ch.bytes = at - start;
            ch.page_end = (int32_t)plan.pages.size();
            ch.unpack_end = (int32_t)plan.unpacks.size();
            plan.chunks.push_back(ch);
            plan.packed += (ch.bytes + 15) & ~15ll;
        }
        row0 += g.num_rows;
    }
    if (row0 != meta.num_rows) return set_error(kUnsupported, "row groups do not add up to the file's rows");
    if (plan.pages.size() > (size_t)INT32_MAX || plan.items > (int64_t)INT32_MAX || plan.n_idx > (int64_t)INT32_MAX ||
        plan.unpacks.size() > (size_t)INT32_MAX)
        return set_error(kUnsupported, "too many pages");
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
    ChunkPlan plan;
    if (int e = plan_chunks(file, n, meta, projections, n_proj, dtypes, optional, plan)) return e;
    std::vector<ParquetPage>& pages = plan.pages;
    const int64_t items = plan.items;

    cudaStream_t st = cudaStreamPerThread;
    keep_pool_memory();
    CopyLane* lane = nullptr;
    if (int e = copy_lane(lane)) return e;
    DevBuf dfile(st), dunpack(st), djobs(st), dpages(st), dstatus(st), ditems(st), dpresent(st), didx(st);
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
    // any other host memory is copied in, chunk by chunk.  Snappy pages are decompressed into the
    // unpack buffer first.
    const uint8_t* direct = device_view(file, n);
    if (!direct)
        if (int e = dfile.alloc((size_t)plan.packed)) return e;
    if (int e = dunpack.alloc((size_t)plan.unpack_bytes)) return e;
    auto file_at = [&](int64_t off, int32_t chunk) -> const uint8_t* {
        if (direct) return direct + off;
        const Chunk& c = plan.chunks[chunk];
        return (const uint8_t*)dfile.p + c.dev_off + (off - c.file_off);
    };
    auto where_at = [&](const PageWhere& w) -> const uint8_t* {
        return w.unpack >= 0 ? (const uint8_t*)dunpack.p + w.unpack : file_at(w.file_off, w.chunk);
    };
    // read in place, a dictionary would be looked up at random over the host link: the
    // dictionaries come into device memory first (one small copy job each, one launch)
    DevBuf ddict(st), dcopies(st);
    std::map<int64_t, int64_t> dict_copy;  // a dictionary's file offset -> its offset in ddict
    std::vector<CopyJob> cjobs;
    if (direct) {
        int64_t dbytes = 0;
        for (size_t k = 0; k < pages.size(); k++) {
            const PageWhere& dw = plan.dict_where[k];
            if (pages[k].dict_count <= 0 || dw.unpack >= 0 || dict_copy.count(dw.file_off)) continue;
            // the copy keeps the source's offset within 16 bytes, so that it moves whole 16-byte words
            const int64_t mis = (int64_t)((uintptr_t)(direct + dw.file_off) & 15);
            dict_copy[dw.file_off] = dbytes + mis;
            const int64_t b = (int64_t)pages[k].dict_count * gdf_dtype_size(dtypes[pages[k].column]);
            cjobs.push_back({direct + dw.file_off, nullptr, b});
            dbytes += ((mis + b + 15) & ~15ll) + 16;
        }
        if (!cjobs.empty()) {
            if (int e = ddict.alloc((size_t)dbytes)) return e;
            for (size_t k = 0; k < pages.size(); k++) {
                const PageWhere& dw = plan.dict_where[k];
                if (pages[k].dict_count <= 0 || dw.unpack >= 0) continue;
                pages[k].dict = (int64_t)(uintptr_t)((char*)ddict.p + dict_copy[dw.file_off]);
            }
            for (CopyJob& cj : cjobs) {
                const int64_t off = (int64_t)(cj.src - direct);
                cj.dst = (uint8_t*)ddict.p + dict_copy[off];
            }
            if (int e = dcopies.alloc(cjobs.size() * sizeof(CopyJob))) return e;
            if (int e = check_cuda(cudaMemcpyAsync(dcopies.p, cjobs.data(), cjobs.size() * sizeof(CopyJob),
                                                   cudaMemcpyHostToDevice, st),
                                   "cudaMemcpyAsync"))
                return e;
            if (int e = check_cuda(launch_copy_jobs((const CopyJob*)dcopies.p, (int32_t)cjobs.size(), st), "dictionary copies"))
                return e;
        }
    }
    for (size_t k = 0; k < pages.size(); k++) {
        pages[k].data = (int64_t)(uintptr_t)where_at(plan.where[k]);
        if (pages[k].dict_count > 0 && !(direct && plan.dict_where[k].unpack < 0))
            pages[k].dict = (int64_t)(uintptr_t)where_at(plan.dict_where[k]);
    }
    std::vector<SnappyJob> jobs(plan.unpacks.size());
    for (size_t k = 0; k < jobs.size(); k++) {
        const Unpack& u = plan.unpacks[k];
        jobs[k].src = file_at(u.src_off, u.chunk);
        jobs[k].dst = (uint8_t*)dunpack.p + u.dst_off;
        jobs[k].src_bytes = (int32_t)u.src_bytes;
        jobs[k].dst_bytes = (int32_t)u.dst_bytes;
        jobs[k].prefix = u.prefix;
    }
    if (int e = djobs.alloc(jobs.size() * sizeof(SnappyJob))) return e;
    if (!jobs.empty() && check_cuda(cudaMemcpyAsync(djobs.p, jobs.data(), jobs.size() * sizeof(SnappyJob),
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
    if (int e = ditems.alloc((size_t)items * 4)) return e;
    cudaMemsetAsync(ditems.p, 0, (size_t)items * 4, st);
    if (int e = dpresent.alloc(pages.size() * 4)) return e;
    cudaMemsetAsync(dpresent.p, 0, pages.size() * 4, st);
    if (int e = didx.alloc((size_t)plan.n_idx * 4)) return e;
    ParquetDecodeParams dp{};
    dp.pages = (ParquetPage*)dpages.p;
    dp.status = (unsigned long long*)dstatus.p;
    dp.item_base = (uint32_t*)ditems.p;
    dp.page_present = (uint32_t*)dpresent.p;
    dp.idx = (uint32_t*)didx.p;
    for (int q = 0; q < n_proj; q++) {
        dp.out[q].data = frame[q].data;
        dp.out[q].valid = (uint32_t*)frame[q].valid;
        dp.out[q].width = gdf_dtype_size(dtypes[q]);
    }
    // the decode of chunks [c0, c1): Snappy pages, level lengths of Snappy v1 pages, levels,
    // dictionary indices, values
    auto decode = [&](size_t c0, size_t c1) -> int {
        const Chunk& a = plan.chunks[c0];
        const Chunk& b = plan.chunks[c1 - 1];
        if (b.unpack_end > a.unpack_begin &&
            check_cuda(launch_snappy_decompress((const SnappyJob*)djobs.p + a.unpack_begin, b.unpack_end - a.unpack_begin,
                                                dp.status, st),
                       "Snappy decompression"))
            return kCudaError;
        if (b.page_end <= a.page_begin) return kSuccess;
        dp.page_lo = a.page_begin;
        dp.page_hi = b.page_end;
        dp.item_lo = pages[a.page_begin].item0;
        dp.item_hi = b.page_end < (int32_t)pages.size() ? pages[b.page_end].item0 : (int32_t)items;
        bool opt = false, dict = false, lens = false;
        for (int32_t k = a.page_begin; k < b.page_end; k++) {
            opt |= pages[k].optional != 0;
            dict |= pages[k].dict_count > 0;
            lens |= pages[k].levels < 0;
        }
        if (lens && check_cuda(launch_parquet_level_lengths(dp, st), "Parquet level lengths")) return kCudaError;
        if (opt && check_cuda(launch_parquet_levels(dp, st), "Parquet definition levels")) return kCudaError;
        if (dict && check_cuda(launch_parquet_dict_indices(dp, st), "Parquet dictionary indices")) return kCudaError;
        return check_cuda(launch_parquet_values(dp, st), "Parquet page values");
    };
    // the copy lane starts after this stream's work so far; on every exit this stream waits for
    // the lane before any buffer is freed
    if (int e = check_cuda(cudaEventRecord(lane->ready, st), "cudaEventRecord")) return e;
    if (int e = check_cuda(cudaStreamWaitEvent(lane->s, lane->ready, 0), "cudaStreamWaitEvent")) return e;
    LaneJoin join{lane, st};
    if (direct) {
        if (!plan.chunks.empty())
            if (int e = decode(0, plan.chunks.size())) return e;
    }
    // Otherwise the chunks go in batches of about kBatchBytes: a batch's chunks are copied on the
    // copy lane's stream while the batch before it is decoded on this one.
    const int64_t kBatchBytes = batch_bytes();
    size_t batch = 0;
    for (size_t c0 = direct ? plan.chunks.size() : 0; c0 < plan.chunks.size(); batch++) {
        size_t c1 = c0;
        int64_t bytes = 0;
        while (c1 < plan.chunks.size() && (c1 == c0 || bytes < kBatchBytes)) {
            const Chunk& c = plan.chunks[c1];
            if (c.bytes > 0 && check_cuda(cudaMemcpyAsync((char*)dfile.p + c.dev_off, file + c.file_off, (size_t)c.bytes,
                                                          cudaMemcpyHostToDevice, lane->s),
                                          "cudaMemcpyAsync"))
                return kCudaError;
            bytes += c.bytes;
            c1++;
        }
        cudaEvent_t copied = nullptr;
        if (int e = lane_event(*lane, batch, &copied)) return e;
        if (int e = check_cuda(cudaEventRecord(copied, lane->s), "cudaEventRecord")) return e;
        if (int e = check_cuda(cudaStreamWaitEvent(st, copied, 0), "cudaStreamWaitEvent")) return e;
        if (int e = decode(c0, c1)) return e;
        c0 = c1;
    }
    std::vector<unsigned long long> status(1 + n_proj, 0);
    if (int e = check_cuda(cudaMemcpyAsync(status.data(), dstatus.p, status.size() * 8, cudaMemcpyDeviceToHost, st),
                           "cudaMemcpyAsync"))
        return e;
    if (int e = check_cuda(cudaStreamSynchronize(st), "Parquet page decode")) return e;
    if (status[0])
        return set_error(kUnsupported, std::to_string(status[0]) + " malformed pages (compressed data, levels, "
                                       "dictionary indices or values that do not decode within their page)");
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
