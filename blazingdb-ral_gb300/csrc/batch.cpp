// batch.cpp — batched execution of many register programs.
//
// The reference runs each program as its own perform_operation call (stream create, program
// upload, launch, synchronise; src/Interpreter/interpreter_cpp.cu:219-286).  A batch runs all
// programs in one persistent kernel whose warps pull (program, warp-tile) work items from a
// device counter, so tables of very different sizes share the GPU in one launch; the launch
// (counter reset + kernel) is captured once as a CUDA graph and replayed.  Each program's tile
// function is relocatable code compiled once per structure (in parallel, cached on disk) and
// linked with a small dispatcher, so a new mix of known programs costs a link, not a compile.
#include "batch.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <thread>

namespace ral {

namespace {

std::mutex g_tune_mu;
struct TuneEntry {
    int J = 0, U = 1, S = 0;
    double ms = 0;
};
std::map<std::string, TuneEntry> g_tune;
bool g_tune_loaded = false;

std::string tune_path() {
    const char* d = std::getenv("RAL_JIT_CACHE_DIR");
    std::string dir;
    if (d && *d) dir = d;
    else {
        const char* home = std::getenv("HOME");
        dir = std::string(home && *home ? home : "/tmp") + "/.cache/ralgpu-jit";
    }
    return dir + "/autotune.json";
}

// The table is a flat JSON object {"key": [J, U, ms, S], ...}; keys contain no quotes.
void load_tune_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    std::ifstream f(tune_path());
    if (!f) return;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string t = ss.str();
    size_t i = 0;
    while ((i = t.find('"', i)) != std::string::npos) {
        const size_t e = t.find('"', i + 1);
        if (e == std::string::npos) break;
        const std::string key = t.substr(i + 1, e - i - 1);
        const size_t lb = t.find('[', e), rb = t.find(']', e);
        if (lb == std::string::npos || rb == std::string::npos) break;
        TuneEntry te;
        const int got = std::sscanf(t.c_str() + lb + 1, "%d , %d , %lf , %d", &te.J, &te.U, &te.ms, &te.S);
        if (got >= 3 && te.J >= 1 && te.J <= 64 && te.U >= 1 && te.U <= 64) {
            if (got < 4) te.S = 0;
            g_tune[key] = te;
        }
        i = rb + 1;
    }
}

void save_tune_locked() {
    const std::string path = tune_path();
    std::ofstream f(path + ".tmp");
    if (!f) return;
    f << "{\n";
    size_t k = 0;
    for (const auto& kv : g_tune) {
        f << "  \"" << kv.first << "\": [" << kv.second.J << ", " << kv.second.U << ", " << kv.second.ms << ", "
          << kv.second.S << "]"
          << (++k < g_tune.size() ? ",\n" : "\n");
    }
    f << "}\n";
    f.close();
    std::rename((path + ".tmp").c_str(), path.c_str());
}

int64_t bucket(int64_t x) {
    int64_t b = 1;
    while (b < x) b <<= 1;
    return b;
}

}  // namespace

// Relative work of a batch entry: rows times a per-row op cost in which the double operations
// that are long instruction sequences (transcendentals, division, power) weigh more.
double work_estimate(const BatchEntry& e) {
    double per_row = 2.0;
    for (const Op& op : e.program.ops) {
        double w = 1.0;
        if (op.unary && op.uop >= BLZ_SIN && op.uop <= BLZ_ATAN) w = 20.0;
        else if (op.unary && (op.uop == BLZ_LN || op.uop == BLZ_LOG)) w = 20.0;
        else if (!op.unary && op.bop == GDF_POW) w = 30.0;
        else if (!op.unary && (op.bop == GDF_DIV || op.bop == GDF_FLOOR_DIV || op.bop == GDF_MOD)) w = 6.0;
        per_row += w;
    }
    return per_row * (double)e.rows;
}

// RAL_BATCH_GRAB: consecutive work items a warp takes per atomic (default 1: measured 121 ms
// against 122 / 124 / 131 / 159 ms at 2 / 4 / 8 / 32 on the 256-program mix, and 15.0 ms against
// 15.9 / 18.0 / 24.0 / 70.6 with tables capped at 1M rows -- smaller grabs end the launch more
// evenly, and one atomic per warp tile is far below the counter's rate)
int batch_grab() {
    const char* e = std::getenv("RAL_BATCH_GRAB");
    const int v = e ? std::atoi(e) : 0;
    return v >= 1 && v <= 64 ? v : 1;
}

int compile_items(const std::vector<GeneratedKernel>& items, std::vector<const std::vector<char>*>& objects,
                  std::string* logs) {
    const size_t n = items.size();
    objects.assign(n, nullptr);
    std::vector<std::string> errs(n), plogs(n);
    std::atomic<size_t> next{0};
    auto work = [&] {
        for (size_t i; (i = next.fetch_add(1)) < n;) objects[i] = jit_object(items[i], errs[i], &plogs[i]);
    };
    unsigned hw = std::thread::hardware_concurrency();
    const size_t nt = std::min<size_t>(n, std::max(1u, std::min(hw ? hw : 4u, 32u)));
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    for (size_t i = 0; i < n; i++) {
        if (logs) *logs += plogs[i];
        if (!objects[i]) return set_error(kJitError, errs[i]);
    }
    return kSuccess;
}

std::string tune_key(const Program& p, int G) {
    // G (widest column), program length bucket, share of F64 register ops, referenced inputs bucket
    int f64ops = 0;
    for (const Op& op : p.ops) f64ops += op.ok == Kind::F64;
    const int nops = (int)p.ops.size();
    const char* fshare = f64ops == 0 ? "none" : 2 * f64ops < nops ? "some" : "most";
    auto ref = p.inputs_referenced();
    int nin = 0;
    for (int c = 0; c < p.n_in; c++) nin += ref[c] ? 1 : 0;
    return "G" + std::to_string(G) + ":ops" + std::to_string(bucket(std::max(1, nops))) + ":f64" + fshare + ":in" +
           std::to_string(bucket(std::max(1, nin)));
}

Shape tuned_shape(const Program& p, int G) {
    Shape s;
    s.G = G;
    s.J = std::max(1, 8 / G);
    s.unroll = 1;
    s.threads = 256;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    load_tune_locked();
    auto it = g_tune.find(tune_key(p, G));
    if (it != g_tune.end()) {
        s.J = it->second.J;
        s.unroll = it->second.U;
        s.soft = it->second.S != 0;
    }
    return s;
}

void record_tuned_shape(const Program& p, int G, int J, int U, bool soft, double ms) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    load_tune_locked();
    TuneEntry te;
    te.J = J;
    te.U = U;
    te.S = soft ? 1 : 0;
    te.ms = ms;
    g_tune[tune_key(p, G)] = te;
    save_tune_locked();
}

Batch::~Batch() {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (d_descs_) cudaFree(d_descs_);
    if (d_prefix_) cudaFree(d_prefix_);
    if (d_fn_) cudaFree(d_fn_);
    if (d_counter_) cudaFree(d_counter_);
}

int64_t Batch::total_rows() const {
    int64_t r = 0;
    for (const auto& e : entries_) r += e->rows;
    return r;
}

int Batch::add(gdf_column* const* outputs, int n_out, gdf_column* const* inputs, int n_in, const ProgramArrays& pa) {
    if (prepared_) return set_error(kInvalidArgument, "batch already prepared");
    auto e = std::make_unique<BatchEntry>();
    if (int rc = build_program(e->program, outputs, n_out, inputs, n_in, pa, false)) return -rc;
    const int64_t n = inputs[0]->size;
    for (int c = 0; c < n_in; c++)
        if (inputs[c]->size < n) return -set_error(kInvalidArgument, "input column shorter than input 0");
    for (int o = 0; o < n_out; o++)
        if (outputs[o]->size < n) return -set_error(kInvalidArgument, "output column shorter than the input");
    for (int c = 0; c < n_in; c++) e->inputs.push_back(*inputs[c]);
    for (int o = 0; o < n_out; o++) e->outputs.push_back(*outputs[o]);
    e->rows = n;
    entries_.push_back(std::move(e));
    return (int)entries_.size() - 1;
}

int Batch::prepare(cudaStream_t st) {
    if (prepared_) return kSuccess;
    if (entries_.empty()) return set_error(kInvalidArgument, "empty batch");
    std::vector<const Program*> progs;
    std::vector<Shape> shapes;
    for (auto& e : entries_) {
        const Program& p = e->program;
        Shape s;
        s.G = 16 / max_width(p);
        bool ok = true;
        auto ref = p.inputs_referenced();
        for (int c = 0; c < p.n_in; c++) {
            if (ref[c] && ((uintptr_t)e->inputs[c].data % ((size_t)s.G * gdf_dtype_size(e->inputs[c].dtype)))) ok = false;
            if (e->inputs[c].valid && ((uintptr_t)e->inputs[c].valid & 3))
                return set_error(kInvalidArgument, "validity masks must be 4-byte aligned");
        }
        for (int o = 0; o < p.n_out; o++) {
            if ((uintptr_t)e->outputs[o].data % ((size_t)s.G * gdf_dtype_size(e->outputs[o].dtype))) ok = false;
            if (e->outputs[o].valid && ((uintptr_t)e->outputs[o].valid & 3))
                return set_error(kInvalidArgument, "validity masks must be 4-byte aligned");
        }
        if (!ok) s.G = 1;
        const int G = s.G;
        s = tuned_shape(p, G);
        if (forced_J_ > 0) {
            s.J = forced_J_;
            s.unroll = forced_U_;
            s.soft = forced_S_;
        }
        e->shape = s;
        e->items = (e->rows + 32LL * s.G * s.J - 1) / (32LL * s.G * s.J);
        progs.push_back(&p);
        shapes.push_back(s);
    }
    // item functions: one per distinct (structure, shape), compiled in parallel, then the dispatcher
    std::vector<GeneratedKernel> items;
    std::map<std::string, int> index_of;
    std::vector<int> fn(entries_.size());
    std::vector<ParamLayout> layouts;
    int stride = 1;
    // Programs run in order of decreasing estimated work (longest-processing-time first), so the
    // launch ends on short programs instead of waiting for one long one to finish.
    std::stable_sort(entries_.begin(), entries_.end(), [](const std::unique_ptr<BatchEntry>& a,
                                                          const std::unique_ptr<BatchEntry>& b) {
        return work_estimate(*a) > work_estimate(*b);
    });
    for (size_t q = 0; q < entries_.size(); q++) {
        GeneratedKernel it = generate_batch_item(entries_[q]->program, entries_[q]->shape);
        layouts.push_back(it.layout);
        stride = std::max(stride, it.layout.total);
        auto f = index_of.find(it.name);
        if (f == index_of.end()) {
            f = index_of.emplace(it.name, (int)items.size()).first;
            items.push_back(std::move(it));
        }
        fn[q] = f->second;
    }
    std::vector<DispatchEntry> names;
    for (const auto& it : items) names.push_back({it.name, false});
    GeneratedKernel disp = generate_batch_dispatch(names, 0, batch_grab());
    items.push_back(disp);
    std::vector<const std::vector<char>*> objects;
    if (int e = compile_items(items, objects, nullptr)) return e;
    std::string err;
    kernel_ = jit_link(disp.name, disp.name, objects, err);
    if (!kernel_) return set_error(kJitError, err);
    kernel_name_ = disp.name;
    stride_ = stride;

    const int NP = (int)entries_.size();
    std::vector<uint64_t> descs((size_t)NP * stride, 0);
    std::vector<long long> prefix(NP + 1, 0);
    for (int q = 0; q < NP; q++) {
        const BatchEntry& e = *entries_[q];
        const ParamLayout& L = layouts[q];
        uint64_t* s = descs.data() + (size_t)q * stride;
        s[L.n_rows] = (uint64_t)e.rows;
        for (int c = 0; c < e.program.n_in; c++) {
            s[L.in_data + c] = (uint64_t)(uintptr_t)e.inputs[c].data;
            s[L.in_valid + c] = (uint64_t)(uintptr_t)e.inputs[c].valid;
        }
        for (int o = 0; o < e.program.n_out; o++) {
            s[L.out_data + o] = (uint64_t)(uintptr_t)e.outputs[o].data;
            s[L.out_valid + o] = (uint64_t)(uintptr_t)e.outputs[o].valid;
        }
        std::vector<uint64_t> slots(L.total, 0);
        fill_scalars(e.program, L, slots);
        for (int k = 0; k < L.total; k++)
            if (slots[k]) s[k] = slots[k];
        prefix[q + 1] = prefix[q] + e.items;
    }
    total_items_ = prefix[NP];
    // the work counter is 32-bit and every warp may overshoot it by one grab
    if (total_items_ > (int64_t)1 << 31) return set_error(kInvalidArgument, "batch too large: more than 2^31 warp tiles");
    if (int e = check_cuda(cudaMalloc(&d_descs_, descs.size() * 8), "cudaMalloc")) return e;
    if (int e = check_cuda(cudaMalloc(&d_prefix_, prefix.size() * 8), "cudaMalloc")) return e;
    if (int e = check_cuda(cudaMalloc(&d_fn_, fn.size() * sizeof(int)), "cudaMalloc")) return e;
    if (int e = check_cuda(cudaMalloc((void**)&d_counter_, sizeof(unsigned int)), "cudaMalloc")) return e;
    cudaMemcpyAsync(d_descs_, descs.data(), descs.size() * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_prefix_, prefix.data(), prefix.size() * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_fn_, fn.data(), fn.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (int e = check_cuda(cudaStreamSynchronize(st), "batch upload")) return e;
    smem_ = batch_dispatch_smem(NP, 0);
    if (smem_ > 48 * 1024 &&
        check_cuda(cudaFuncSetAttribute((const void*)kernel_->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_),
                   "cudaFuncSetAttribute"))
        return kCudaError;

    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)kernel_->kernel, 256, smem_) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
    }
    per_sm_ = std::max(1, per_sm);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, (const void*)kernel_->kernel) == cudaSuccess) registers_ = fa.numRegs;
    else cudaGetLastError();
    grid_ = std::max(1, sms * std::max(1, per_sm));
    const int64_t warps_needed = (total_items_ + batch_grab() - 1) / batch_grab();
    grid_ = (int)std::max<int64_t>(1, std::min<int64_t>(grid_, (warps_needed + 7) / 8));

    // capture the launch (counter reset + kernel) once
    cudaStream_t cap = nullptr;
    if (int e = check_cuda(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "cudaStreamCreate")) return e;
    int rc = check_cuda(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    if (!rc) rc = launch(cap);
    cudaGraph_t g = nullptr;
    const int rc2 = check_cuda(cudaStreamEndCapture(cap, &g), "cudaStreamEndCapture");
    if (!rc) rc = rc2;
    if (!rc) {
        graph_ = g;
        rc = check_cuda(cudaGraphInstantiate(&graph_exec_, graph_, 0), "cudaGraphInstantiate");
    }
    cudaStreamDestroy(cap);
    if (rc) return rc;
    prepared_ = true;
    return kSuccess;
}

int Batch::debug_source(bool compile, std::string& source, std::string& log) const {
    std::vector<GeneratedKernel> items;
    std::map<std::string, int> seen;
    for (const auto& e : entries_) {
        Shape sh = tuned_shape(e->program, 16 / max_width(e->program));
        GeneratedKernel it = generate_batch_item(e->program, sh);
        if (seen.emplace(it.name, 1).second) items.push_back(std::move(it));
    }
    std::vector<DispatchEntry> names;
    for (const auto& it : items) names.push_back({it.name, false});
    items.push_back(generate_batch_dispatch(names, 0, batch_grab()));
    source.clear();
    for (const auto& it : items) source += "// ---- " + it.name + "\n" + it.source + "\n";
    if (compile) {
        std::vector<const std::vector<char>*> objects;
        if (int e = compile_items(items, objects, &log)) return e;
        std::string err, llog;
        size_t bytes = 0;
        if (!jit_link_only(objects, &bytes, &llog, err)) return set_error(kJitError, err);
        log += llog;
    }
    return kSuccess;
}

int Batch::launch(cudaStream_t st) {
    if (int e = check_cuda(cudaMemsetAsync(d_counter_, 0, sizeof(unsigned int), st), "cudaMemsetAsync")) return e;
    const void* descs = d_descs_;
    const void* prefix = d_prefix_;
    int np = (int)entries_.size();
    unsigned int* counter = d_counter_;
    long long total = total_items_;
    const void* fn = d_fn_;
    const void* base = nullptr;
    int stride = stride_;
    void* args[] = {&descs, &stride, &prefix, &base, &fn, &np, &counter, &total};
    return check_cuda(cudaLaunchKernel((const void*)kernel_->kernel, dim3(grid_), dim3(256), args, smem_, st),
                      "launch of the batch kernel");
}

int Batch::run(cudaStream_t st, bool use_graph) {
    if (!prepared_) {
        if (int e = prepare(st)) return e;
    }
    if (total_items_ == 0) return kSuccess;
    if (use_graph) {
        if (int e = check_cuda(cudaGraphLaunch(graph_exec_, st), "cudaGraphLaunch")) return e;
    } else {
        if (int e = launch(st)) return e;
    }
    note_launch();
    return kSuccess;
}

}  // namespace ral
