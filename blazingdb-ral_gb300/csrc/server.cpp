// server.cpp — request loop over HBM-resident tables with continuous batching.
//
// The reference evaluates one query at a time: each LogicalFilter / LogicalProject step is its
// own sequence of synchronous kernel calls (src/CalciteInterpreter.cpp:509-573 and 311-336).
// Here a scheduler thread keeps up to max_waves persistent launches in flight; each launch
// carries every request admitted since the previous one, as (request, chunk) work items of the
// fused filter + project chunk function of its query.
#include "server.h"

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>

#include "batch.h"
#include "engine.h"

namespace ral {

namespace {

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Waiting credit of the wave order: a request that has waited 1 ms ranks as if it had 10M rows
// fewer left (about the rows the GPU scans in that time), so that large requests are not starved.
constexpr double kAgeRowsPerSecond = 1e10;

// Item shape of a query: vector width from the widest column, chunks of RAL_SERVER_CHUNK rows
// (default 2048; 1024 measured the same), predicate unroll 2, and the FP64 instructions
// (RAL_SERVER_SOFT_FP=1 for the integer-pipe double operations: measured 1656 requests/s at
// capacity against 1756 with the FP64 instructions).
Shape query_shape(const FilterPlan& plan, bool aligned16) {
    Shape sh;
    sh.G = aligned16 ? 16 / filter_max_width(plan.spec) : 1;
    const char* c = std::getenv("RAL_SERVER_CHUNK");
    const int rows = c && std::atoi(c) >= 32 && std::atoi(c) <= 8192 ? std::atoi(c) : 2048;
    sh.J = std::max(1, rows / (32 * sh.G));
    sh.threads = 256;
    sh.min_blocks = 1;
    sh.unroll = 2;
    sh.stage = false;
    const char* f = std::getenv("RAL_SERVER_SOFT_FP");
    sh.soft = f && std::string(f) == "1";
    return sh;
}

// Register cap of the served chunk functions and their dispatcher (RAL_SERVER_MAXRREG, default
// 64: four 256-thread blocks per SM).
int server_max_registers() {
    const char* e = std::getenv("RAL_SERVER_MAXRREG");
    const int v = e ? std::atoi(e) : 0;
    return v >= 32 && v <= 255 ? v : 64;
}

// Layout of one request's allocation: scratch | output masks | output data (each 256-aligned),
// so that everything that must start at zero is one memset.
struct RequestLayout {
    size_t scratch_bytes = 0, zero_bytes = 0, total = 0;
    std::vector<size_t> valid_off, data_off;
};

RequestLayout request_layout(const ServerQuery& q, int64_t rows) {
    RequestLayout L;
    const FilterPlan& p = *q.plan;
    const int NO = (int)p.out_dtypes.size();
    L.scratch_bytes = (size_t)std::max<int64_t>(filter_scratch_header(NO) + q.chunks, q.scratch_words) * 8;
    size_t off = round_up(L.scratch_bytes, 256);
    for (int k = 0; k < NO; k++) {
        L.valid_off.push_back(p.out_valid[k] ? off : (size_t)-1);
        if (p.out_valid[k]) off += round_up((size_t)gdf_valid_allocation_size(rows), 256);
    }
    L.zero_bytes = off;
    for (int k = 0; k < NO; k++) {
        L.data_off.push_back(off);
        off += round_up((size_t)std::max<int64_t>(rows, 1) * gdf_dtype_size(p.out_dtypes[k]), 256);
    }
    L.total = off;
    return L;
}

}  // namespace

Server::Server(size_t budget_bytes, int max_waves, int max_wave_requests, int64_t wave_rows)
    : budget_(budget_bytes), max_waves_(std::max(1, std::min(max_waves, 8))),
      max_wave_requests_(std::max(1, std::min(max_wave_requests, 4096))) {
    wave_rows_ = wave_rows > 0 ? wave_rows : ((int64_t)32 << 20);
    // RAL_SERVER_SLICE_DIV: a request takes at most wave_rows / this of one wave (default 2;
    // measured at 90% load: 4 gives p50 / p99 3.6 / 41.6 ms, 1 gives 6.3 / 31.3 ms)
    const char* sd = std::getenv("RAL_SERVER_SLICE_DIV");
    slice_div_ = sd && std::atoi(sd) >= 1 && std::atoi(sd) <= 64 ? std::atoi(sd) : 2;
    // RAL_SERVER_SOLO_ROWS: requests over tables of at least this many rows run the standalone
    // fused kernel alone on a wave (default half a wave; 0 turns it off)
    const char* so = std::getenv("RAL_SERVER_SOLO_ROWS");
    solo_rows_ = so ? std::atoll(so) : wave_rows_ / 2;
    t0_ = 0;
    t0_ = now();
}

Server::~Server() {
    stop();
    for (auto& w : waves_) {
        if (w.done) cudaEventDestroy(w.done);
        if (w.stream) cudaStreamDestroy(w.stream);
        if (w.d_desc) cudaFree(w.d_desc);
        if (w.h_desc) cudaFreeHost(w.h_desc);
        if (w.h_head) cudaFreeHost(w.h_head);
    }
    for (auto& kv : requests_)
        if (kv.second->scratch) cudaFree(kv.second->scratch);
}

double Server::now() const {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count() - t0_;
}

int Server::add_table(gdf_column* const* cols, int ncols, int* table_id) {
    if (!cols || ncols <= 0 || !table_id) return set_error(kInvalidArgument, "null argument");
    ServerTable t;
    for (int c = 0; c < ncols; c++) {
        if (!cols[c]) return set_error(kInvalidArgument, "null column");
        if (cols[c]->size != cols[0]->size) return set_error(kInvalidArgument, "table columns differ in size");
        t.cols.push_back(*cols[c]);
        t.bytes += (size_t)cols[c]->size * gdf_dtype_size(cols[c]->dtype);
        if (cols[c]->valid) t.bytes += gdf_valid_allocation_size(cols[c]->size);
    }
    t.rows = cols[0]->size;
    std::lock_guard<std::mutex> lock(mu_);
    if (tables_bytes_ + t.bytes >= budget_) return set_error(kInvalidArgument, "resident tables exceed the budget");
    tables_bytes_ += t.bytes;
    tables_.push_back(std::move(t));
    *table_id = (int)tables_.size() - 1;
    return kSuccess;
}

int Server::add_query(int table_id, const char* filter_q, const char* project_q, int* query_id) {
    std::lock_guard<std::mutex> lock(mu_);
    if (table_id < 0 || table_id >= (int)tables_.size()) return set_error(kInvalidArgument, "unknown table");
    ServerTable& t = tables_[table_id];
    std::vector<gdf_column*> frame;
    bool al = true;
    for (auto& c : t.cols) {
        frame.push_back(&c);
        if ((uintptr_t)c.data % 16) al = false;
    }
    auto q = std::make_unique<ServerQuery>();
    q->table = table_id;
    if (int e = plan_filter_project(frame.data(), (int)frame.size(), filter_q, project_q, q->plan)) return e;
    const Shape sh = query_shape(*q->plan, al);
    q->item = generate_filter_kernel(q->plan->spec, sh, true);
    q->item.max_registers = server_max_registers();
    // at least one chunk, so that an empty table's request still runs (and finishes) once
    q->chunks = std::max<int64_t>(1, (t.rows + filter_tile_rows(sh) - 1) / filter_tile_rows(sh));
    if (solo_rows_ > 0 && max_waves_ > 1) {
        // the standalone kernel is compiled when the server starts (all queries at once, on
        // threads); its scratch is bounded here by one status word per 32 rows (its smallest chunk)
        q->large = t.rows >= solo_rows_;
        q->filter_text = filter_q;
        q->project_text = project_q;
        q->scratch_words = filter_scratch_header((int)q->plan->out_dtypes.size()) + (t.rows + 31) / 32 + 1;
    }
    q->reserve = request_layout(*q, t.rows).total;
    if (q->plan->out_dtypes.size() > 64) return set_error(kUnsupported, "more than 64 projected columns");
    if (tables_bytes_ + q->reserve > budget_)
        return set_error(kInvalidArgument, "one request of this query exceeds the budget");
    queries_.push_back(std::move(q));
    *query_id = (int)queries_.size() - 1;
    return kSuccess;
}

int Server::query_outputs(int query_id, std::vector<gdf_dtype>& dtypes, std::vector<bool>& valid) const {
    std::lock_guard<std::mutex> lock(mu_);
    if (query_id < 0 || query_id >= (int)queries_.size()) return set_error(kInvalidArgument, "unknown query");
    dtypes = queries_[query_id]->plan->out_dtypes;
    valid = queries_[query_id]->plan->out_valid;
    return kSuccess;
}

// One translation unit and one dispatcher entry per distinct item function: queries whose
// filter and projection generate the same code (same column types, masks and operators, any
// table) share one function, because the linker accepts each extern symbol once.  Sets each
// query's dispatcher index.
void Server::collect_items(std::vector<GeneratedKernel>& tus, std::vector<DispatchEntry>& entries, int& stride,
                           int& smem) {
    std::unordered_map<std::string, int> index;
    stride = 1;
    smem = 0;
    for (auto& q : queries_) {
        auto it = index.find(q->item.name);
        if (it == index.end()) {
            it = index.emplace(q->item.name, (int)entries.size()).first;
            tus.push_back(q->item);
            entries.push_back({q->item.name, true});
        }
        q->fn = it->second;
        stride = std::max(stride, q->item.layout.total);
        smem = std::max(smem, q->item.item_smem_words);
    }
}

// Compiles the item functions of all queries and links the dispatcher; (re)allocates the
// wave buffers.  Called with mu_ held and no wave in flight.
// The standalone kernels of the queries that have none yet, compiled on host threads.
int Server::prepare_solo_kernels() {
    std::vector<ServerQuery*> todo;
    for (auto& q : queries_)
        if (!q->solo && !q->filter_text.empty()) todo.push_back(q.get());
    if (todo.empty()) return kSuccess;
    std::atomic<size_t> next{0};
    std::atomic<int> failed{0};
    std::mutex err_mu;
    std::string first_err;
    auto work = [&] {
        cudaSetDevice(device_);
        for (size_t i; (i = next++) < todo.size();) {
            ServerQuery& q = *todo[i];
            ServerTable& t = tables_[q.table];
            std::vector<gdf_column*> frame;
            for (auto& c : t.cols) frame.push_back(&c);
            // stand-in outputs: only dtypes and mask presence matter to the plan
            const int NO = (int)q.plan->out_dtypes.size();
            std::vector<gdf_column> stand(NO);
            std::vector<gdf_column*> souts(NO);
            for (int o = 0; o < NO; o++) {
                stand[o] = gdf_column{};
                stand[o].dtype = q.plan->out_dtypes[o];
                stand[o].valid = q.plan->out_valid[o] ? (gdf_valid_type*)(uintptr_t)256 : nullptr;
                stand[o].size = (gdf_size_type)t.rows;
                souts[o] = &stand[o];
            }
            const void* h = nullptr;
            if (prepare_standalone_filter(frame.data(), (int)frame.size(), q.filter_text.c_str(), q.project_text.c_str(),
                                          souts.data(), NO, &h) ||
                standalone_scratch_words(h, t.rows) > q.scratch_words) {
                std::lock_guard<std::mutex> lock(err_mu);
                if (!failed++) first_err = last_error();
                continue;
            }
            q.solo = h;
        }
    };
    // a string literal missing from a category dictionary rewrites its column while planning:
    // with category columns the kernels are prepared one at a time
    bool categories = false;
    for (const auto& t : tables_)
        for (const auto& c : t.cols) categories |= c.dtype == GDF_STRING_CATEGORY;
    const int nt = categories ? 1
                              : (int)std::min<size_t>(todo.size(),
                                                      std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
    std::vector<std::thread> pool;
    for (int k = 1; k < nt; k++) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    if (failed) return set_error(kJitError, "standalone filter kernel of a served query: " + first_err);
    return kSuccess;
}

int Server::ensure_linked() {
    if (linked_queries_ == (int)queries_.size() && kernel_) return kSuccess;
    if (queries_.empty()) return set_error(kInvalidArgument, "no queries");
    if (int e = prepare_solo_kernels()) return e;
    std::vector<GeneratedKernel> tus;
    std::vector<DispatchEntry> entries;
    int stride = 1, smem = 0;
    collect_items(tus, entries, stride, smem);
    GeneratedKernel disp = generate_batch_dispatch(entries, smem, 1);
    disp.max_registers = server_max_registers();
    tus.push_back(disp);
    std::vector<const std::vector<char>*> objs;
    if (int e = compile_items(tus, objs, nullptr)) return e;
    std::string err;
    const CompiledKernel* k = jit_link(disp.name, disp.name, objs, err);
    if (!k) return set_error(kJitError, err);
    const size_t dsmem = batch_dispatch_smem(max_wave_requests_, smem);
    if (dsmem > 48 * 1024 &&
        check_cuda(cudaFuncSetAttribute((const void*)k->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem),
                   "cudaFuncSetAttribute"))
        return kCudaError;
    int sms = 1, per_sm = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k->kernel, 256, dsmem) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
    }
    grid_ = sms * std::max(1, per_sm);
    kernel_ = k;
    stride_ = stride;
    smem_words_ = smem;
    linked_queries_ = (int)queries_.size();
    // wave buffers: descs | prefix | base | fn | counter
    const size_t M = (size_t)max_wave_requests_;
    const size_t bytes =
        round_up(M * stride_ * 8, 16) + round_up((M + 1) * 8, 16) + round_up(M * 8, 16) + round_up(M * 4, 16) + 16;
    if (waves_.empty()) waves_.resize(max_waves_);
    for (auto& w : waves_) {
        if (!w.stream && check_cuda(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking), "cudaStreamCreate"))
            return kCudaError;
        if (!w.done && check_cuda(cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming), "cudaEventCreate"))
            return kCudaError;
        if (w.desc_bytes < bytes) {
            if (w.d_desc) cudaFree(w.d_desc);
            if (w.h_desc) cudaFreeHost(w.h_desc);
            w.d_desc = w.h_desc = nullptr;
            if (check_cuda(cudaMalloc(&w.d_desc, bytes), "cudaMalloc") ||
                check_cuda(cudaMallocHost(&w.h_desc, bytes), "cudaMallocHost"))
                return kCudaError;
            w.desc_bytes = bytes;
        }
        if (!w.h_head) {
            // scratch headers: at most 3 + 64 outputs words per request
            if (check_cuda(cudaMallocHost(&w.h_head, M * 67 * 8), "cudaMallocHost")) return kCudaError;
        }
    }
    return kSuccess;
}

int Server::debug_compile(std::string& log) {
    std::lock_guard<std::mutex> lock(mu_);
    if (queries_.empty()) return set_error(kInvalidArgument, "no queries");
    std::vector<GeneratedKernel> tus;
    std::vector<DispatchEntry> entries;
    int stride = 1, smem = 0;
    collect_items(tus, entries, stride, smem);
    tus.push_back(generate_batch_dispatch(entries, smem, 1));
    tus.back().max_registers = server_max_registers();
    std::vector<const std::vector<char>*> objs;
    if (int e = compile_items(tus, objs, &log)) return e;
    std::string err, llog;
    size_t bytes = 0;
    if (!jit_link_only(objs, &bytes, &llog, err)) return set_error(kJitError, err);
    log += llog;
    return kSuccess;
}

int Server::start() {
    std::lock_guard<std::mutex> lock(mu_);
    if (started_) return kSuccess;
    cudaGetDevice(&device_);
    // keep freed request memory in the pool instead of returning it to the driver each time
    keep_pool_memory();
    if (int e = ensure_linked()) return e;
    started_ = true;
    stop_ = false;
    thread_ = std::thread([this] { loop(); });
    return kSuccess;
}

int Server::submit(int query_id, bool keep, int64_t* request_id) {
    std::lock_guard<std::mutex> lock(mu_);
    if (!started_) return set_error(kInvalidArgument, "server not started");
    if (fatal_) return set_error(fatal_, fatal_msg_);
    if (query_id < 0 || query_id >= (int)queries_.size()) return set_error(kInvalidArgument, "unknown query");
    auto r = std::make_unique<ServerRequest>();
    r->id = next_id_++;
    r->query = query_id;
    r->keep = keep;
    r->t_submit = now();
    if (request_id) *request_id = r->id;
    pending_.push_back(r->id);
    requests_.emplace(r->id, std::move(r));
    stats_.submitted++;
    cv_.notify_one();
    return kSuccess;
}

int Server::launch_wave(Wave& w, const std::vector<int64_t>& reqs, const std::vector<int64_t>& take) {
    const int NP = (int)reqs.size();
    const size_t M = (size_t)max_wave_requests_;
    char* h = (char*)w.h_desc;
    uint64_t* descs = (uint64_t*)h;
    const size_t off_prefix = round_up(M * stride_ * 8, 16);
    const size_t off_base = off_prefix + round_up((M + 1) * 8, 16);
    const size_t off_fn = off_base + round_up(M * 8, 16);
    const size_t off_counter = off_fn + round_up(M * 4, 16);
    long long* prefix = (long long*)(h + off_prefix);
    long long* base = (long long*)(h + off_base);
    int* fn = (int*)(h + off_fn);
    std::memset(h + off_counter, 0, 16);
    prefix[0] = 0;
    const double t = now();
    w.last.assign(NP, 0);
    for (int k = 0; k < NP; k++) {
        ServerRequest& r = *requests_[reqs[k]];
        ServerQuery& q = *queries_[r.query];
        ServerTable& tb = tables_[q.table];
        if (r.next_chunk == 0) {
            if (int e = start_request(r, w.stream)) return e;
            r.t_launch = t;
        }
        if (r.slots.empty()) {
            std::vector<gdf_column*> frame;
            for (auto& c : tb.cols) frame.push_back(&c);
            filter_fill_slots(*q.plan, q.item, frame.data(), tb.rows, r.out_data.data(), r.out_valid.data(), r.scratch,
                              r.slots);
        }
        std::memcpy(descs + (size_t)k * stride_, r.slots.data(), r.slots.size() * 8);
        prefix[k + 1] = prefix[k] + take[k];
        base[k] = r.next_chunk;
        fn[k] = q.fn;
        r.next_chunk += take[k];
        w.last[k] = r.next_chunk >= q.chunks;
        r.in_wave = true;
    }
    const long long total = prefix[NP];
    char* d = (char*)w.d_desc;
    cudaMemcpyAsync(d, h, (size_t)NP * stride_ * 8, cudaMemcpyHostToDevice, w.stream);
    cudaMemcpyAsync(d + off_prefix, h + off_prefix, (size_t)(NP + 1) * 8, cudaMemcpyHostToDevice, w.stream);
    cudaMemcpyAsync(d + off_base, h + off_base, (size_t)NP * 8, cudaMemcpyHostToDevice, w.stream);
    cudaMemcpyAsync(d + off_fn, h + off_fn, (size_t)NP * 4, cudaMemcpyHostToDevice, w.stream);
    cudaMemcpyAsync(d + off_counter, h + off_counter, 16, cudaMemcpyHostToDevice, w.stream);
    const void* a_descs = d;
    int a_stride = stride_;
    const void* a_prefix = d + off_prefix;
    const void* a_base = d + off_base;
    const void* a_fn = d + off_fn;
    int a_np = NP;
    unsigned int* a_counter = (unsigned int*)(d + off_counter);
    long long a_total = total;
    void* args[] = {&a_descs, &a_stride, &a_prefix, &a_base, &a_fn, &a_np, &a_counter, &a_total};
    const int grid = (int)std::max<long long>(1, std::min<long long>(grid_, (total + 7) / 8));
    const size_t smem = batch_dispatch_smem(NP, smem_words_);
    if (total > 0) {
        if (int e = check_cuda(cudaLaunchKernel((const void*)kernel_->kernel, dim3(grid), dim3(256), args, smem, w.stream),
                               "launch of the served dispatcher"))
            return e;
        note_launch();
    }
    // scratch headers of the requests that finish in this wave: error flag, kept rows, valid counts
    uint64_t* hh = (uint64_t*)w.h_head;
    for (int k = 0; k < NP; k++) {
        if (!w.last[k]) continue;
        ServerRequest& r = *requests_[reqs[k]];
        const int NO = (int)queries_[r.query]->plan->out_dtypes.size();
        cudaMemcpyAsync(hh + (size_t)k * 67, r.scratch, (size_t)filter_scratch_header(NO) * 8, cudaMemcpyDeviceToHost,
                        w.stream);
    }
    if (int e = check_cuda(cudaEventRecord(w.done, w.stream), "cudaEventRecord")) return e;
    w.reqs = reqs;
    w.take = take;
    w.busy = true;
    w.t_launch = t;
    if (inflight_ == 0) busy_since_ = t;
    inflight_++;
    stats_.waves++;
    stats_.max_wave_requests = std::max<int64_t>(stats_.max_wave_requests, NP);
    return kSuccess;
}

// A request's first launch: its outputs and scratch, zeroed where the kernels expect it.
int Server::start_request(ServerRequest& r, cudaStream_t st) {
    ServerQuery& q = *queries_[r.query];
    ServerTable& tb = tables_[q.table];
    const RequestLayout L = request_layout(q, tb.rows);
    void* mem = nullptr;
    if (int e = check_cuda(cudaMallocAsync(&mem, L.total, st), "cudaMallocAsync")) return e;
    cudaMemsetAsync(mem, 0, L.zero_bytes, st);
    r.scratch = mem;
    const int NO = (int)q.plan->out_dtypes.size();
    r.out_data.assign(NO, nullptr);
    r.out_valid.assign(NO, nullptr);
    for (int o = 0; o < NO; o++) {
        r.out_data[o] = (char*)mem + L.data_off[o];
        if (L.valid_off[o] != (size_t)-1) r.out_valid[o] = (char*)mem + L.valid_off[o];
    }
    return kSuccess;
}

// A large request alone on a wave: the standalone fused filter + project kernel over its table,
// its header (error word, kept count, valid counts) copied to the wave's first header slot.
int Server::launch_solo(Wave& w, int64_t id) {
    ServerRequest& r = *requests_[id];
    ServerQuery& q = *queries_[r.query];
    ServerTable& tb = tables_[q.table];
    const double t = now();
    if (int e = start_request(r, w.stream)) return e;
    r.t_launch = t;
    const int NO = (int)q.plan->out_dtypes.size();
    std::vector<gdf_column*> frame;
    for (auto& c : tb.cols) frame.push_back(&c);
    std::vector<gdf_column> outs(NO);
    std::vector<gdf_column*> pouts(NO);
    for (int o = 0; o < NO; o++) {
        outs[o] = gdf_column{};
        outs[o].dtype = q.plan->out_dtypes[o];
        outs[o].data = r.out_data[o];
        outs[o].valid = (gdf_valid_type*)r.out_valid[o];
        outs[o].size = (gdf_size_type)tb.rows;
        pouts[o] = &outs[o];
    }
    if (int e = enqueue_standalone_filter(q.solo, frame.data(), pouts.data(), r.scratch,
                                          (unsigned long long*)w.h_head, w.stream))
        return e;
    if (int e = check_cuda(cudaEventRecord(w.done, w.stream), "cudaEventRecord")) return e;
    r.next_chunk = q.chunks;
    r.in_wave = true;
    w.reqs = {id};
    w.take = {q.chunks};
    w.last.assign(1, 1);
    w.busy = true;
    w.solo = true;
    w.t_launch = t;
    if (inflight_ == 0) busy_since_ = t;
    inflight_++;
    solo_inflight_++;
    stats_.waves++;
    stats_.solo++;
    stats_.max_wave_requests = std::max<int64_t>(stats_.max_wave_requests, 1);
    return kSuccess;
}

// Bookkeeping of a wave that is no longer in flight.
void Server::wave_ended(Wave& w) {
    w.reqs.clear();
    w.busy = false;
    if (w.solo) {
        w.solo = false;
        solo_inflight_--;
    }
    inflight_--;
}

void Server::finish_wave(Wave& w) {
    const double t = now();
    const uint64_t* hh = (const uint64_t*)w.h_head;
    for (size_t k = 0; k < w.reqs.size(); k++) {
        ServerRequest& r = *requests_[w.reqs[k]];
        r.in_wave = false;
        if (!w.last[k]) continue;
        ServerQuery& q = *queries_[r.query];
        const uint64_t* head = hh + k * 67;
        const int NO = (int)q.plan->out_dtypes.size();
        r.t_done = t;
        stats_.queue_s += r.t_launch - r.t_submit;
        stats_.run_s += t - r.t_launch;
        if (head[1]) {
            r.status = kTimeout;
            r.rows_out = -1;
        } else {
            r.rows_out = (int64_t)head[2];
            r.null_counts.assign(NO, 0);
            for (int o = 0; o < NO; o++)
                if (q.plan->out_valid[o]) r.null_counts[o] = r.rows_out - (int64_t)head[3 + o];
        }
        if (!r.keep) {
            cudaFreeAsync(r.scratch, w.stream);
            r.scratch = nullptr;
            r.out_data.clear();
            r.out_valid.clear();
            reserved_ -= q.reserve;  // kept outputs stay reserved until release
        }
        r.done = true;
        active_.erase(std::find(active_.begin(), active_.end(), r.id));
        stats_.completed++;
    }
    wave_ended(w);
    if (inflight_ == 0 && busy_since_ >= 0) {
        stats_.busy_s += t - busy_since_;
        busy_since_ = -1;
    }
    done_cv_.notify_all();
}

void Server::loop() {
    cudaSetDevice(device_);
    std::unique_lock<std::mutex> lk(mu_);
    double last_busy = now();
    while (true) {
        for (auto& w : waves_) {
            if (!w.busy) continue;
            const cudaError_t q = cudaEventQuery(w.done);
            if (q == cudaSuccess) finish_wave(w);
            else if (q != cudaErrorNotReady) {
                fatal_ = kCudaError;
                fatal_msg_ = std::string("served wave failed: ") + cudaGetErrorString(q);
                cudaGetLastError();
                for (int64_t id : w.reqs) {
                    requests_[id]->status = kCudaError;
                    requests_[id]->done = true;
                }
                wave_ended(w);
                done_cv_.notify_all();
            }
        }
        if (stop_ && pending_.empty() && active_.empty() && inflight_ == 0) break;
        Wave* free_w = nullptr;
        for (auto& w : waves_)
            if (!w.busy) { free_w = &w; break; }
        const bool need_link = linked_queries_ < (int)queries_.size();
        if (free_w && !fatal_ && (!pending_.empty() || !active_.empty()) && (!need_link || inflight_ == 0)) {
            int rc = need_link ? ensure_linked() : 0;
            // admission (FIFO): while the working set stays under the budget
            const size_t cap = budget_ - tables_bytes_;
            while (!rc && !pending_.empty()) {
                ServerRequest& r = *requests_[pending_.front()];
                const size_t need = queries_[r.query]->reserve;
                if (reserved_ + need > cap) break;  // wait for memory to free up
                reserved_ += need;
                active_.push_back(r.id);
                pending_.pop_front();
            }
            stats_.peak_reserved = std::max(stats_.peak_reserved, reserved_);
            // A request not yet started runs alone on the standalone kernel when its table is large
            // (on at most all but one of the waves: one stays for the batched small requests), or
            // when nothing else waits to be launched (a batch of one gains nothing from the
            // dispatcher).
            if (!rc) {
                int64_t solo_id = -1, waiting = 0;
                for (int64_t id : active_) {
                    const ServerRequest& r = *requests_[id];
                    if (r.in_wave) continue;
                    waiting++;
                    const ServerQuery& q = *queries_[r.query];
                    if (solo_id < 0 && r.next_chunk == 0 && q.solo && q.large && solo_inflight_ < max_waves_ - 1)
                        solo_id = id;
                }
                if (solo_id < 0 && waiting == 1 && pending_.empty()) {
                    for (int64_t id : active_) {
                        const ServerRequest& r = *requests_[id];
                        if (!r.in_wave && r.next_chunk == 0 && queries_[r.query]->solo) solo_id = id;
                    }
                }
                if (solo_id >= 0) {
                    rc = launch_solo(*free_w, solo_id);
                    if (rc) {
                        fatal_ = rc;
                        fatal_msg_ = last_error();
                        requests_[solo_id]->status = rc;
                        requests_[solo_id]->done = true;
                        done_cv_.notify_all();
                    }
                    continue;
                }
            }
            // the wave: requests not in flight, fewest rows left (less a waiting credit) first,
            // each with at most a quarter of the wave, up to wave_rows_ rows
            std::vector<int64_t> reqs, take;
            std::vector<std::pair<double, int64_t>> cand;  // (priority, id)
            const double tnow = now();
            for (int64_t id : active_) {
                const ServerRequest& r = *requests_[id];
                if (r.in_wave) continue;
                const ServerQuery& q = *queries_[r.query];
                if (q.solo && q.large && r.next_chunk == 0) continue;  // waits for a solo wave
                const double left = (double)(q.chunks - r.next_chunk) * (double)filter_tile_rows(q.item.shape);
                cand.push_back({left - (tnow - r.t_submit) * kAgeRowsPerSecond, id});
            }
            std::sort(cand.begin(), cand.end());
            const int64_t slice = std::max<int64_t>(1, wave_rows_ / slice_div_);
            int64_t rows = 0;
            for (auto& c : cand) {
                if ((int)reqs.size() >= max_wave_requests_ || rows >= wave_rows_) break;
                const ServerRequest& r = *requests_[c.second];
                const ServerQuery& q = *queries_[r.query];
                const int64_t rpc = filter_tile_rows(q.item.shape);
                const int64_t left = q.chunks - r.next_chunk;
                const int64_t cap_rows = std::min(slice, wave_rows_ - rows);
                const int64_t n = std::max<int64_t>(1, std::min<int64_t>(left, (cap_rows + rpc - 1) / rpc));
                reqs.push_back(c.second);
                take.push_back(n);
                rows += n * rpc;
            }
            if (!rc && !reqs.empty()) rc = launch_wave(*free_w, reqs, take);
            if (rc) {
                fatal_ = rc;
                fatal_msg_ = last_error();
                for (int64_t id : reqs) {
                    requests_[id]->status = rc;
                    requests_[id]->done = true;
                }
                done_cv_.notify_all();
            }
        }
        if (inflight_ > 0 || now() - last_busy < 0.005) {
            // waves in flight, or idle for less than 5 ms: poll (a yield, not a sleep, so that
            // completions and new requests are noticed within microseconds)
            if (inflight_ > 0 || !pending_.empty()) last_busy = now();
            lk.unlock();
            std::this_thread::yield();
            lk.lock();
        } else {
            cv_.wait_for(lk, std::chrono::milliseconds(2));
            last_busy = now();
        }
    }
}

int Server::wait(int64_t id, double timeout_s, int64_t* rows_out, double* latency_s) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = requests_.find(id);
    if (it == requests_.end()) return set_error(kInvalidArgument, "unknown request");
    ServerRequest& r = *it->second;
    const bool ok = done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return r.done; });
    if (!ok) return set_error(kTimeout, "request not done within the timeout");
    if (r.status) return set_error(r.status, fatal_msg_.empty() ? "request failed" : fatal_msg_);
    if (rows_out) *rows_out = r.rows_out;
    if (latency_s) *latency_s = r.t_done - r.t_submit;
    return kSuccess;
}

int Server::result(int64_t id, gdf_column* out, int n_out) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = requests_.find(id);
    if (it == requests_.end()) return set_error(kInvalidArgument, "unknown request");
    ServerRequest& r = *it->second;
    if (!r.done || r.status) return set_error(kInvalidArgument, "request not done");
    if (!r.keep || !r.scratch) return set_error(kInvalidArgument, "request outputs were not kept");
    const ServerQuery& q = *queries_[r.query];
    if (n_out != (int)q.plan->out_dtypes.size()) return set_error(kInvalidArgument, "wrong output count");
    for (int o = 0; o < n_out; o++) {
        out[o] = gdf_column{};
        out[o].data = r.out_data[o];
        out[o].valid = (gdf_valid_type*)r.out_valid[o];
        out[o].size = (gdf_size_type)r.rows_out;
        out[o].dtype = q.plan->out_dtypes[o];
        out[o].null_count = (gdf_size_type)r.null_counts[o];
    }
    return kSuccess;
}

int Server::release(int64_t id) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = requests_.find(id);
    if (it == requests_.end()) return set_error(kInvalidArgument, "unknown request");
    if (!it->second->done) return set_error(kInvalidArgument, "request still running");
    if (it->second->scratch) {
        cudaFree(it->second->scratch);
        reserved_ -= queries_[it->second->query]->reserve;
    }
    requests_.erase(it);
    return kSuccess;
}

int Server::run_trace(int n, const int32_t* queries, const double* arrival_s, double* latency_s, int64_t* rows_out,
                      double* makespan_s) {
    std::vector<int64_t> ids(n);
    const double t_start = now();
    for (int k = 0; k < n; k++) {
        const double due = t_start + arrival_s[k];
        for (;;) {
            const double dt = due - now();
            if (dt <= 0) break;
            if (dt > 200e-6) std::this_thread::sleep_for(std::chrono::duration<double>(dt - 100e-6));
            else std::this_thread::yield();
        }
        if (int e = submit(queries[k], false, &ids[k])) return e;
    }
    double last = t_start;
    for (int k = 0; k < n; k++) {
        int64_t rows = 0;
        if (int e = wait(ids[k], 600.0, &rows, nullptr)) return e;
        std::lock_guard<std::mutex> lock(mu_);
        ServerRequest& r = *requests_[ids[k]];
        // latency from the scheduled arrival, so that any lag of the submitting thread counts
        if (latency_s) latency_s[k] = r.t_done - (t_start + arrival_s[k]);
        if (rows_out) rows_out[k] = rows;
        last = std::max(last, r.t_done);
        requests_.erase(ids[k]);
    }
    if (makespan_s) *makespan_s = last - (t_start + (n ? arrival_s[0] : 0.0));
    return kSuccess;
}

int Server::stop() {
    {
        std::lock_guard<std::mutex> lock(mu_);
        if (!started_) return kSuccess;
        stop_ = true;
        cv_.notify_all();
    }
    if (thread_.joinable()) thread_.join();
    std::lock_guard<std::mutex> lock(mu_);
    started_ = false;
    return kSuccess;
}

ServerStats Server::stats() const {
    std::lock_guard<std::mutex> lock(mu_);
    return stats_;
}

}  // namespace ral
