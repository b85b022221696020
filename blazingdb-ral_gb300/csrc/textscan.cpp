// textscan.cpp — a table scan over delimited text fused with its LogicalFilter.
//
// The reference scans a CSV table in CalciteInterpreter.cpp:745-767 (BindableTableScan: the
// `projects=[...]` list picks the file columns) through csv_parser::parse
// (src/io/data_parser/CSVParser.cpp:176-233, cudf's CSV reader), and a LogicalFilter above the
// scan then evaluates its condition over the scanned frame and compacts it
// (CalciteInterpreter.cpp:509-573).  Here the text stays in device memory and the two run as one:
// a line index (three small kernels: terminators per tile, a scan, their positions), then one
// generated kernel that parses the predicate's fields of every line, evaluates the predicate,
// finds each chunk's output offset by look-back and parses and stores the projected fields of the
// kept lines only.  Field rules: csrc/textscan.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "codegen.h"
#include "engine.h"
#include "frontend.h"
#include "jit.h"
#include "kernels.h"
#include "program.h"
#include "ral/ral_c.h"
#include "textscan.h"

namespace ral {

namespace {

// A stream-ordered device allocation freed on scope exit.
struct StreamBuffer {
    void* p = nullptr;
    cudaStream_t st = nullptr;
    explicit StreamBuffer(cudaStream_t s) : st(s) {}
    StreamBuffer(const StreamBuffer&) = delete;
    StreamBuffer& operator=(const StreamBuffer&) = delete;
    ~StreamBuffer() {
        if (p) cudaFreeAsync(p, st);
    }
    int alloc(size_t bytes) { return check_cuda(cudaMallocAsync(&p, std::max<size_t>(bytes, 16), st), "cudaMallocAsync"); }
};

bool scanned_dtype(gdf_dtype t) {
    switch (t) {
    case GDF_INT8: case GDF_INT16: case GDF_INT32: case GDF_INT64: case GDF_FLOAT32: case GDF_FLOAT64:
    case GDF_DATE32: case GDF_DATE64:
        return true;
    default:
        return false;
    }
}

// The positions of every line terminator of data[0, n) (device memory, on st) and the line count.
struct LineIndex {
    StreamBuffer ends;
    int64_t nterm = 0;
    int64_t lines = 0;
    explicit LineIndex(cudaStream_t st) : ends(st) {}
};

int build_line_index(const char* data, int64_t n, char term, cudaStream_t st, LineIndex& li) {
    if (n <= 0) return kSuccess;
    const int64_t tiles = text_tiles(n);
    StreamBuffer counts(st), offsets(st);
    if (int e = counts.alloc((size_t)tiles * 4)) return e;
    if (int e = offsets.alloc((size_t)(tiles + 1) * 8)) return e;
    if (int e = check_cuda(launch_text_term_counts(data, n, term, (uint32_t*)counts.p, st), "line terminators")) return e;
    if (int e = check_cuda(launch_exclusive_scan_u32((const uint32_t*)counts.p, tiles, (unsigned long long*)offsets.p, st),
                           "line terminator scan"))
        return e;
    // the terminator count and the last byte decide the line count and the index's size
    thread_local unsigned long long* h = nullptr;
    if (!h && check_cuda(cudaMallocHost((void**)&h, 16), "cudaMallocHost")) return kCudaError;
    if (int e = check_cuda(cudaMemcpyAsync(h, (unsigned long long*)offsets.p + tiles, 8, cudaMemcpyDeviceToHost, st),
                           "cudaMemcpyAsync"))
        return e;
    if (int e = check_cuda(cudaMemcpyAsync((char*)(h + 1), data + n - 1, 1, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync"))
        return e;
    if (int e = check_cuda(cudaStreamSynchronize(st), "line index")) return e;
    li.nterm = (int64_t)h[0];
    const char last = *(const char*)(h + 1);
    li.lines = li.nterm + (last != term ? 1 : 0);
    if (int e = li.ends.alloc((size_t)li.nterm * 8)) return e;
    return check_cuda(launch_text_term_positions(data, n, term, (const unsigned long long*)offsets.p, (long long*)li.ends.p, st),
                      "line terminator positions");
}

// A compiled scan kernel with its predicate program (the program's scalars fill the launch).
struct PreparedScan {
    Program pred;
    bool have_pred = false;
    TextScanSpec spec;
    GeneratedKernel gk;
    const CompiledKernel* k = nullptr;
};
std::mutex g_scan_mu;
std::map<std::string, std::unique_ptr<PreparedScan>> g_scans;

Shape text_scan_shape() {
    Shape s;
    s.J = 8;  // 256 lines per look-back chunk
    s.threads = 256;
    s.min_blocks = 4;
    apply_shape_tune(s, std::getenv("RAL_SCAN_TUNE") ? std::getenv("RAL_SCAN_TUNE") : "");
    return s;
}

// The spec and generated kernel of a scan (no compilation).
int build_scan(const std::vector<gdf_dtype>& dtypes, const std::vector<int>& file_cols, const char* filter_q,
               PreparedScan& scan) {
    PreparedScan* ps = &scan;
    ps->spec.dtypes = dtypes;
    ps->spec.file_cols = file_cols;
    if (filter_q) {
        const std::string cond = named_expression(filter_q, "condition");
        if (cond.empty()) return set_error(kParseError, "no condition=[...] in the LogicalFilter");
        const int NP = (int)dtypes.size();
        // stand-in columns of the scanned frame: any field may be null
        std::vector<gdf_column> frame(NP);
        std::vector<gdf_column*> pf(NP);
        for (int q = 0; q < NP; q++) {
            frame[q] = gdf_column{};
            frame[q].dtype = dtypes[q];
            frame[q].valid = (gdf_valid_type*)(uintptr_t)64;  // only its presence matters here
            frame[q].size = 1;
            frame[q].null_count = 1;
            pf[q] = &frame[q];
        }
        ExpressionPlan ep = plan_expression(cond, NP);
        if (ep.clone)
            return set_error(kUnsupported, "a bare \"$k\" condition over a scanned text column is not supported");
        gdf_column stencil{};
        stencil.dtype = GDF_INT8;
        stencil.valid = (gdf_valid_type*)(uintptr_t)64;
        stencil.size = 1;
        gdf_column* souts[1] = {&stencil};
        std::vector<gdf_column*> ins;
        for (int c : ep.input_columns) ins.push_back(pf[c]);
        ProgramArrays pa{ep.pv.left.data(), ep.pv.right.data(), ep.pv.outs.data(), (int32_t)ep.pv.left.size(),
                         ep.pv.final_pos.data(), ep.pv.bops.data(), ep.pv.uops.data(), ep.pv.lscalars.data(),
                         ep.pv.rscalars.data()};
        if (int e = build_program(ps->pred, souts, 1, ins.data(), (int)ins.size(), pa, false)) return e;
        ps->have_pred = true;
        ps->spec.predicate = &ps->pred;
        ps->spec.predicate_cols = ep.input_columns;
    }
    ps->gk = generate_text_scan_kernel(ps->spec, text_scan_shape());
    return kSuccess;
}

int prepare_scan(const std::vector<gdf_dtype>& dtypes, const std::vector<int>& file_cols, const char* filter_q,
                 const PreparedScan** out) {
    const Shape sh = text_scan_shape();
    std::string key = std::string(filter_q ? filter_q : "") + "|";
    for (size_t q = 0; q < dtypes.size(); q++) key += std::to_string((int)dtypes[q]) + "@" + std::to_string(file_cols[q]) + ",";
    key += "|J" + std::to_string(sh.J) + "T" + std::to_string(sh.threads) + "B" + std::to_string(sh.min_blocks);
    {
        std::lock_guard<std::mutex> lock(g_scan_mu);
        auto it = g_scans.find(key);
        if (it != g_scans.end()) {
            *out = it->second.get();
            return kSuccess;
        }
    }
    auto ps = std::make_unique<PreparedScan>();
    if (int e = build_scan(dtypes, file_cols, filter_q, *ps)) return e;
    std::string err;
    ps->k = jit_get(ps->gk, err);
    if (!ps->k) return set_error(kJitError, err);
    std::lock_guard<std::mutex> lock(g_scan_mu);
    auto res = g_scans.emplace(key, std::move(ps));
    *out = res.first->second.get();
    return kSuccess;
}

}  // namespace

int text_scan_rows(const char* data, int64_t n, char term, int32_t skip_rows, int64_t* rows) {
    if (!rows || n < 0 || skip_rows < 0 || (n > 0 && !data)) return set_error(kInvalidArgument, "bad argument");
    *rows = 0;
    if (n == 0) return kSuccess;
    cudaStream_t st = cudaStreamPerThread;
    LineIndex li(st);
    if (int e = build_line_index(data, n, term, st, li)) return e;
    StreamBuffer cnt(st);
    if (int e = cnt.alloc(8)) return e;
    cudaMemsetAsync(cnt.p, 0, 8, st);
    if (int e = check_cuda(launch_text_present_count(data, n, (const long long*)li.ends.p, li.nterm, li.lines, skip_rows,
                                                     (unsigned long long*)cnt.p, st),
                           "line count"))
        return e;
    unsigned long long h = 0;
    if (int e = check_cuda(cudaMemcpyAsync(&h, cnt.p, 8, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync")) return e;
    if (int e = check_cuda(cudaStreamSynchronize(st), "line count")) return e;
    *rows = (int64_t)h;
    return kSuccess;
}

// The scanned frame's dtypes and file columns from the file schema and the projections.
int scan_columns(const int32_t* file_dtypes, int32_t n_file, const int32_t* projections, int32_t n_proj,
                 std::vector<gdf_dtype>& dtypes, std::vector<int>& file_cols) {
    if (!file_dtypes || n_file <= 0 || !projections || n_proj <= 0) return set_error(kInvalidArgument, "bad argument");
    if (n_proj > 64) return set_error(kUnsupported, "more than 64 projected columns");
    dtypes.resize(n_proj);
    file_cols.resize(n_proj);
    for (int q = 0; q < n_proj; q++) {
        if (projections[q] < 0 || projections[q] >= n_file) return set_error(kInvalidArgument, "projection out of range");
        file_cols[q] = projections[q];
        dtypes[q] = (gdf_dtype)file_dtypes[projections[q]];
        if (!scanned_dtype(dtypes[q]))
            return set_error(kUnsupported, "column " + std::to_string(projections[q]) + ": the text scan reads integer, "
                                           "floating-point and date columns");
    }
    return kSuccess;
}

int text_scan_source(const int32_t* file_dtypes, int32_t n_file, const int32_t* projections, int32_t n_proj,
                     const char* filter_q, bool compile, std::string& source, std::string& log) {
    std::vector<gdf_dtype> dtypes;
    std::vector<int> file_cols;
    if (int e = scan_columns(file_dtypes, n_file, projections, n_proj, dtypes, file_cols)) return e;
    PreparedScan ps;
    if (int e = build_scan(dtypes, file_cols, filter_q, ps)) return e;
    source = std::string(jit_prelude()) + "\n" + ps.gk.source;
    if (compile) {
        std::string err;
        size_t bytes = 0;
        if (!jit_compile_only(ps.gk, &bytes, &log, err)) {
            log = err;
            return set_error(kJitError, err);
        }
    }
    return kSuccess;
}

namespace {

// Checks the out columns against the scanned dtypes; their smallest size is the capacity.
int check_outs(const std::vector<gdf_dtype>& dtypes, gdf_column* const* outs, int64_t* cap) {
    *cap = INT64_MAX;
    for (size_t q = 0; q < dtypes.size(); q++) {
        gdf_column* o = outs[q];
        if (!o) return set_error(kInvalidArgument, "null out column");
        if (o->dtype != dtypes[q]) return set_error(kInvalidArgument, "out column " + std::to_string(q) + " has the wrong dtype");
        if (!o->valid || ((uintptr_t)o->valid & 3)) return set_error(kInvalidArgument, "out columns need a 4-byte aligned mask");
        if (o->size > 0 && !o->data) return set_error(kInvalidArgument, "out column without data");
        *cap = std::min<int64_t>(*cap, o->size);
    }
    return kSuccess;
}

// One scan launch over data[0, n) (device memory): its kept rows go to rows row0 .. of the
// outputs (whose masks are zeroed), at most cap of them; adds the rows kept and each output's
// valid rows to kept / valid.  Synchronous on st.
int scan_piece(const PreparedScan& ps, const char* data, int64_t n, char delim, char term, int32_t skip_rows,
               gdf_column* const* outs, int NP, int64_t row0, int64_t cap, cudaStream_t st, int64_t& kept,
               std::vector<int64_t>& valid) {
    LineIndex li(st);
    if (int e = build_line_index(data, n, term, st, li)) return e;
    const GeneratedKernel& gk = ps.gk;
    const ParamLayout& L = gk.layout;
    const int64_t chunks = (li.lines + text_scan_chunk_lines(gk.shape) - 1) / text_scan_chunk_lines(gk.shape);
    if (chunks == 0) return kSuccess;
    const int64_t header = text_scan_header(NP);
    StreamBuffer scratch(st);
    if (int e = scratch.alloc((size_t)(header + chunks) * 8)) return e;
    cudaMemsetAsync(scratch.p, 0, (size_t)(header + chunks) * 8, st);
    // the outputs seen from the word holding row0: row (row0 & 31) + j is kept row j
    const int64_t obase = row0 & 31;
    std::vector<uint64_t> slots(L.total, 0);
    slots[0] = (uint64_t)li.lines;
    slots[1] = (uint64_t)(uintptr_t)data;
    slots[2] = (uint64_t)n;
    slots[3] = (uint64_t)(uintptr_t)li.ends.p;
    slots[4] = (uint64_t)li.nterm;
    slots[5] = (uint64_t)skip_rows;
    slots[6] = (uint64_t)(unsigned char)delim;
    slots[7] = (uint64_t)std::max<int64_t>(cap, 0);
    slots[8] = (uint64_t)obase;
    for (int q = 0; q < NP; q++) {
        const int64_t w = gdf_dtype_size(outs[q]->dtype);
        slots[L.out_data + q] = (uint64_t)(uintptr_t)((char*)outs[q]->data + (row0 - obase) * w);
        slots[L.out_valid + q] = (uint64_t)(uintptr_t)((uint32_t*)outs[q]->valid + (row0 >> 5));
    }
    slots[L.scratch] = (uint64_t)(uintptr_t)scratch.p;
    if (ps.have_pred) fill_scalars(ps.pred, L, slots);
    // the header comes back into page-locked memory: a copy into pageable memory would wait
    // behind the host-to-device copies of a streamed scan
    thread_local unsigned long long* h = nullptr;
    if (!h && check_cuda(cudaMallocHost((void**)&h, 8 * 72), "cudaMallocHost")) return kCudaError;
    const int grid = launch_blocks(*ps.k, gk.shape.threads, text_scan_chunk_lines(gk.shape) * (gk.shape.threads / 32),
                                   li.lines);
    void* args[] = {slots.data()};
    if (int e = check_cuda(cudaLaunchKernel((const void*)ps.k->kernel, dim3(grid), dim3(gk.shape.threads), args, 0, st),
                           "launch of the text scan kernel"))
        return e;
    note_launch();
    if (int e = check_cuda(cudaMemcpyAsync(h, scratch.p, (size_t)header * 8, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync"))
        return e;
    if (int e = check_cuda(cudaStreamSynchronize(st), "text scan kernel")) return e;
    if (h[1]) return set_error(kTimeout, "text scan look-back wait gave up");
    if (h[3 + NP])
        return set_error(kUnsupported, std::to_string(h[3 + NP]) + " decimal fields outside the exactly rounded range "
                                       "(more than 19 significant digits, above 2^53 or a power of ten beyond 1e22)");
    if (h[4 + NP]) return set_error(kInvalidArgument, "the out columns hold fewer rows than the scan keeps");
    kept += (int64_t)h[2];
    for (int q = 0; q < NP; q++) valid[q] += (int64_t)h[3 + q];
    return kSuccess;
}

void set_outputs(gdf_column* const* outs, int NP, int64_t kept, const std::vector<int64_t>& valid, gdf_size_type* n_out) {
    for (int q = 0; q < NP; q++) {
        outs[q]->size = (gdf_size_type)kept;
        outs[q]->null_count = (gdf_size_type)(kept - valid[q]);
    }
    *n_out = (gdf_size_type)kept;
}

// Text handed over in host memory goes to the device in pieces of about this many bytes (whole
// lines; RAL_SCAN_PIECE_BYTES overrides), each scanned while the next ones are copied.
int64_t piece_bytes() {
    const char* e = std::getenv("RAL_SCAN_PIECE_BYTES");
    const long long v = e ? std::atoll(e) : 0;
    return v > 0 ? (int64_t)v : ((int64_t)64 << 20);
}

}  // namespace

int text_scan_filter(const char* data, int64_t n, char delim, char term, int32_t skip_rows, const int32_t* file_dtypes,
                     int32_t n_file, const int32_t* projections, int32_t n_proj, const char* filter_q,
                     gdf_column* const* outs, gdf_size_type* n_out) {
    if (n < 0 || skip_rows < 0 || (n > 0 && !data) || !outs || !n_out) return set_error(kInvalidArgument, "bad argument");
    if (delim == term) return set_error(kInvalidArgument, "the delimiter and the line terminator are the same byte");
    std::vector<gdf_dtype> dtypes;
    std::vector<int> file_cols;
    if (int e = scan_columns(file_dtypes, n_file, projections, n_proj, dtypes, file_cols)) return e;
    int64_t cap = 0;
    if (int e = check_outs(dtypes, outs, &cap)) return e;
    const PreparedScan* ps = nullptr;
    if (int e = prepare_scan(dtypes, file_cols, filter_q, &ps)) return e;
    const int NP = n_proj;
    cudaStream_t st = cudaStreamPerThread;
    keep_pool_memory();
    for (int q = 0; q < NP; q++)
        if (cap > 0) cudaMemsetAsync(outs[q]->valid, 0, (size_t)((cap + 31) / 32) * 4, st);
    int64_t kept = 0;
    std::vector<int64_t> valid(NP, 0);
    if (int e = scan_piece(*ps, data, n, delim, term, skip_rows, outs, NP, 0, cap, st, kept, valid)) return e;
    set_outputs(outs, NP, kept, valid, n_out);
    return kSuccess;
}

int text_scan_filter_host(const char* text, int64_t n, char delim, char term, int32_t skip_rows,
                          const int32_t* file_dtypes, int32_t n_file, const int32_t* projections, int32_t n_proj,
                          const char* filter_q, gdf_column* const* outs, gdf_size_type* n_out) {
    if (n < 0 || skip_rows < 0 || (n > 0 && !text) || !outs || !n_out) return set_error(kInvalidArgument, "bad argument");
    if (delim == term) return set_error(kInvalidArgument, "the delimiter and the line terminator are the same byte");
    std::vector<gdf_dtype> dtypes;
    std::vector<int> file_cols;
    if (int e = scan_columns(file_dtypes, n_file, projections, n_proj, dtypes, file_cols)) return e;
    int64_t cap = 0;
    if (int e = check_outs(dtypes, outs, &cap)) return e;
    const PreparedScan* ps = nullptr;
    if (int e = prepare_scan(dtypes, file_cols, filter_q, &ps)) return e;
    const int NP = n_proj;
    // the skipped lines are passed over here: every piece starts at a line
    int64_t off = 0;
    for (int32_t k = 0; k < skip_rows && off < n; k++) {
        const void* t = std::memchr(text + off, term, (size_t)(n - off));
        off = t ? (int64_t)((const char*)t - text) + 1 : n;
    }
    // pieces of whole lines: each ends just after a terminator (the last at the end of the text).
    // A piece is copied from the 256-byte boundary at or before its first line (copies from
    // unaligned host addresses run slower, and the kernels read aligned text 16 bytes at a time);
    // the lines before its first one there all end inside it and are skipped by the scan.
    const int64_t P = piece_bytes();
    struct Piece {
        int64_t from, to, skip;
    };
    std::vector<Piece> pieces;
    int64_t biggest = 0;
    for (int64_t s0 = off; s0 < n;) {
        int64_t e0 = std::min(n, s0 + P);
        if (e0 < n) {
            const void* t = std::memchr(text + e0 - 1, term, (size_t)(n - (e0 - 1)));
            e0 = t ? (int64_t)((const char*)t - text) + 1 : n;
        }
        const int64_t a = s0 & ~(int64_t)255;
        int64_t skip = 0;
        for (int64_t p = a; p < s0; p++) skip += text[p] == term;
        pieces.push_back({a, e0, skip});
        biggest = std::max(biggest, e0 - a);
        s0 = e0;
    }
    cudaStream_t st = cudaStreamPerThread;
    keep_pool_memory();
    for (int q = 0; q < NP; q++)
        if (cap > 0) cudaMemsetAsync(outs[q]->valid, 0, (size_t)((cap + 31) / 32) * 4, st);
    int64_t kept = 0;
    std::vector<int64_t> valid(NP, 0);
    if (pieces.empty()) {
        set_outputs(outs, NP, kept, valid, n_out);
        return kSuccess;
    }
    // three piece buffers: two copies run ahead of the scan
    const int NB = (int)std::min<size_t>(3, pieces.size());
    std::vector<std::unique_ptr<StreamBuffer>> bufs;
    for (int b = 0; b < NB; b++) {
        bufs.emplace_back(new StreamBuffer(st));
        if (int e = bufs.back()->alloc((size_t)biggest)) return e;
    }
    CopyLane* lane = nullptr;
    if (int e = copy_lane(lane)) return e;
    if (int e = check_cuda(cudaEventRecord(lane->ready, st), "cudaEventRecord")) return e;
    if (int e = check_cuda(cudaStreamWaitEvent(lane->s, lane->ready, 0), "cudaStreamWaitEvent")) return e;
    LaneJoin join{lane, st};  // before the buffers are freed, this stream waits for every copy
    auto copy = [&](size_t k) -> int {
        const int64_t s0 = pieces[k].from, bytes = pieces[k].to - pieces[k].from;
        if (int e = check_cuda(cudaMemcpyAsync(bufs[k % NB]->p, text + s0, (size_t)bytes, cudaMemcpyHostToDevice, lane->s),
                               "cudaMemcpyAsync"))
            return e;
        cudaEvent_t ev = nullptr;
        if (int e = lane_event(*lane, k, &ev)) return e;
        return check_cuda(cudaEventRecord(ev, lane->s), "cudaEventRecord");
    };
    for (size_t k = 0; k + 1 < (size_t)NB; k++)
        if (int e = copy(k)) return e;
    for (size_t k = 0; k < pieces.size(); k++) {
        // the buffer of piece k + NB - 1 held piece k - 1, whose scan has finished
        if (k + NB - 1 < pieces.size())
            if (int e = copy(k + NB - 1)) return e;
        cudaEvent_t ev = nullptr;
        if (int e = lane_event(*lane, k, &ev)) return e;
        if (int e = check_cuda(cudaStreamWaitEvent(st, ev, 0), "cudaStreamWaitEvent")) return e;
        if (int e = scan_piece(*ps, (const char*)bufs[k % NB]->p, pieces[k].to - pieces[k].from, delim, term,
                               (int32_t)pieces[k].skip, outs, NP, kept, cap - kept, st, kept, valid))
            return e;
    }
    set_outputs(outs, NP, kept, valid, n_out);
    return kSuccess;
}

}  // namespace ral
