// engine.cpp — perform_operation: validate, specialise, launch.
//
// Replaces src/Interpreter/interpreter_cpp.cu:219-286.  The reference creates
// a stream, sizes the grid with an occupancy if-chain, allocates temp space,
// copies the program with 18 host-to-device copies and synchronises, per call.
// Here the program is baked into a cached kernel, the column pointers and
// literals travel as one kernel parameter block, and nothing is allocated.
#include "engine.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>

#include "softfp.cuh"

namespace ral {

namespace {
std::atomic<long long> g_launches{0};
thread_local std::string t_error;
thread_local int t_error_code = 0;
}  // namespace

int set_error(int code, const std::string& msg) {
    t_error = msg;
    t_error_code = code;
    return code;
}
const char* last_error() { return t_error.c_str(); }

int check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return kSuccess;
    return set_error(kCudaError, std::string(what) + ": " + cudaGetErrorString(e));
}

void note_launch(int count) { g_launches += count; }
long long launch_count() { return g_launches.load(); }

Config& config() {
    static Config c = [] {
        Config x;
        const char* v = std::getenv("RAL_FLOAT_LITERAL_COMPAT");
        x.float_literal_compat = v && v[0] == '1';
        return x;
    }();
    return c;
}

Shape eval_shape(const Program& p) {
    Shape s = default_shape(p);
    // RAL_EVAL_TUNE: shape overrides for the eval kernels ("J=4,B=3,T=128")
    static const std::string tune = [] {
        const char* e = std::getenv("RAL_EVAL_TUNE");
        return std::string(e ? e : "");
    }();
    if (!tune.empty()) apply_shape_tune(s, tune);
    return s;
}

int build_program(Program& p, gdf_column* const* outputs, int n_out, gdf_column* const* inputs, int n_in,
                  const ProgramArrays& pa, bool ignore_null_count) {
    if (n_in <= 0 || inputs == nullptr) return set_error(kInvalidArgument, "no input columns");
    if (n_out <= 0 || outputs == nullptr) return set_error(kInvalidArgument, "no output columns");
    if (pa.n_ops < 0) return set_error(kInvalidArgument, "negative operation count");
    if (pa.n_ops > 0 && (!pa.left || !pa.right || !pa.outs || !pa.bops || !pa.uops || !pa.lscalars || !pa.rscalars))
        return set_error(kInvalidArgument, "program arrays must not be null");
    if (!pa.final_positions) return set_error(kInvalidArgument, "final_output_positions must not be null");
    std::vector<ColumnDesc> ins(n_in);
    for (int c = 0; c < n_in; c++) {
        const gdf_column* col = inputs[c];
        if (!col) return set_error(kInvalidArgument, "null input column");
        ins[c].dtype = col->dtype;
        ins[c].has_valid = col->valid != nullptr;
        ins[c].nulls_possible = col->valid != nullptr && (ignore_null_count || col->null_count != 0);
    }
    std::vector<gdf_dtype> out_types(n_out);
    std::vector<bool> out_valid(n_out);
    for (int o = 0; o < n_out; o++) {
        if (!outputs[o]) return set_error(kInvalidArgument, "null output column");
        out_types[o] = outputs[o]->dtype;
        out_valid[o] = outputs[o]->valid != nullptr;
    }
    p.float_literal_compat = config().float_literal_compat;
    std::string err;
    if (!p.build(ins, out_types, out_valid, pa.left, pa.right, pa.outs, pa.n_ops, pa.final_positions, pa.bops,
                 pa.uops, pa.lscalars, pa.rscalars, err))
        return set_error(kUnsupported, err);
    return kSuccess;
}

void fill_scalars(const Program& p, const ParamLayout& L, std::vector<uint64_t>& slots) {
    for (size_t k = 0; k < p.ops.size(); k++) {
        if (L.lscalar_slot[k] >= 0) slots[L.lscalar_slot[k]] = p.ops[k].lscalar;
        if (L.rscalar_slot[k] >= 0) slots[L.rscalar_slot[k]] = p.ops[k].rscalar;
        if (k < L.rdiv_slot.size() && L.rdiv_slot[k] >= 0) {
            const RalDivider v = ral_sf_make_divider((long long)p.ops[k].rscalar);
            slots[L.rdiv_slot[k]] = (uint64_t)v.mult;
            slots[L.rdiv_slot[k] + 1] = (uint64_t)v.shift_mode;
        }
    }
}

namespace {

struct DeviceInfo {
    int sms = 0;             // 0: not read yet
    bool pool_kept = false;  // keep_pool_memory ran
};
std::mutex g_dev_mu;
std::unordered_map<int, DeviceInfo> g_devs;
std::unordered_map<std::string, int> g_occupancy;  // kernel name + device -> blocks/SM

}  // namespace

int device_sms() {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_dev_mu);
    DeviceInfo& d = g_devs[dev];
    if (d.sms > 0) return d.sms;
    cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    if (d.sms <= 0) d.sms = 1;
    return d.sms;
}

void keep_pool_memory() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lock(g_dev_mu);
    DeviceInfo& d = g_devs[dev];
    if (d.pool_kept) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    d.pool_kept = true;
}

int copy_lane(CopyLane*& out) {
    int dev = 0;
    if (int e = check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return e;
    static thread_local std::map<int, CopyLane> lanes;
    CopyLane& l = lanes[dev];
    if (!l.s && check_cuda(cudaStreamCreateWithFlags(&l.s, cudaStreamNonBlocking), "cudaStreamCreate")) return kCudaError;
    if (!l.ready && check_cuda(cudaEventCreateWithFlags(&l.ready, cudaEventDisableTiming), "cudaEventCreate"))
        return kCudaError;
    out = &l;
    return kSuccess;
}

int lane_event(CopyLane& lane, size_t k, cudaEvent_t* ev) {
    while (lane.events.size() <= k) {
        cudaEvent_t e = nullptr;
        if (check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate")) return kCudaError;
        lane.events.push_back(e);
    }
    *ev = lane.events[k];
    return kSuccess;
}

int blocks_per_sm(const CompiledKernel& k, int threads) {
    int dev = 0;
    cudaGetDevice(&dev);
    const std::string key = k.name + "@" + std::to_string(dev) + "/" + std::to_string(threads) + "/" +
                            std::to_string(k.dyn_smem);
    {
        std::lock_guard<std::mutex> lock(g_dev_mu);
        auto it = g_occupancy.find(key);
        if (it != g_occupancy.end()) return it->second;
    }
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, (const void*)k.kernel, threads, (size_t)k.dyn_smem) !=
        cudaSuccess) {
        cudaGetLastError();
        b = 1;
    }
    if (b < 1) b = 1;
    std::lock_guard<std::mutex> lock(g_dev_mu);
    g_occupancy[key] = b;
    return b;
}

namespace {

bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

// Key of the generated-kernel cache: program structure + launch shape.
std::mutex g_gen_mu;
std::unordered_map<std::string, GeneratedKernel> g_generated;

const GeneratedKernel& generated_eval(const Program& p, const Shape& s) {
    const std::string key = p.structure_key() + "#" + std::to_string(s.G) + "/" + std::to_string(s.J) + "/" +
                            std::to_string(s.threads) + "/" + std::to_string(s.min_blocks);
    std::lock_guard<std::mutex> lock(g_gen_mu);
    auto it = g_generated.find(key);
    if (it != g_generated.end()) return it->second;
    auto res = g_generated.emplace(key, generate_eval_kernel(p, s));
    return res.first->second;
}

}  // namespace

namespace {
std::atomic<int> g_timing{-1};  // -1: not read from the environment yet
std::atomic<int64_t> g_t_calls{0}, g_t_prep{0}, g_t_enq{0}, g_t_wait{0}, g_t_dev{0};  // nanoseconds
thread_local std::chrono::steady_clock::time_point t_start, t_prepared;
}  // namespace

bool call_timing_enabled() {
    int v = g_timing.load(std::memory_order_relaxed);
    if (v < 0) {
        const char* e = std::getenv("RAL_CALL_TIMING");
        v = (e && e[0] == '1') ? 1 : 0;
        int expect = -1;
        g_timing.compare_exchange_strong(expect, v);
        v = g_timing.load();
    }
    return v == 1;
}

void call_timing_start() {
    if (call_timing_enabled()) t_start = t_prepared = std::chrono::steady_clock::now();
}

void call_timing_mark_prepared() {
    if (call_timing_enabled()) t_prepared = std::chrono::steady_clock::now();
}

void call_timing_add(double enqueue_us, double wait_us, double device_us) {
    if (!call_timing_enabled()) return;
    const double prep = std::chrono::duration<double, std::micro>(t_prepared - t_start).count();
    g_t_calls.fetch_add(1);
    g_t_prep.fetch_add((int64_t)(prep * 1e3));
    g_t_enq.fetch_add((int64_t)(enqueue_us * 1e3));
    g_t_wait.fetch_add((int64_t)(wait_us * 1e3));
    g_t_dev.fetch_add((int64_t)(device_us * 1e3));
}

int call_timing_query(bool enable, bool reset, int64_t* calls, double* us4) {
    g_timing.store(enable ? 1 : 0);
    if (calls) *calls = g_t_calls.load();
    if (us4) {
        const double c = std::max<int64_t>(1, g_t_calls.load());
        us4[0] = g_t_prep.load() / 1e3 / c;
        us4[1] = g_t_enq.load() / 1e3 / c;
        us4[2] = g_t_wait.load() / 1e3 / c;
        us4[3] = g_t_dev.load() / 1e3 / c;
    }
    if (reset) {
        g_t_calls = 0;
        g_t_prep = 0;
        g_t_enq = 0;
        g_t_wait = 0;
        g_t_dev = 0;
    }
    return kSuccess;
}

namespace {
std::mutex g_err_mu;
std::unordered_map<int, unsigned long long*> g_err_words;
}  // namespace

// A word per device that staged kernels set when a bounded wait gave up (allocated once, zeroed).
unsigned long long* device_error_word() {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_err_mu);
    auto it = g_err_words.find(dev);
    if (it != g_err_words.end()) return it->second;
    unsigned long long* w = nullptr;
    if (cudaMalloc((void**)&w, sizeof(unsigned long long)) != cudaSuccess) return nullptr;
    cudaMemset(w, 0, sizeof(unsigned long long));
    cudaDeviceSynchronize();
    g_err_words[dev] = w;
    return w;
}

// Reads and clears the device's error word after a synchronisation: kTimeout when a staged
// kernel's wait gave up since the last check.
int take_device_error(cudaStream_t st) {
    unsigned long long* w = device_error_word();
    if (!w) return kSuccess;
    unsigned long long h = 0;
    if (int e = check_cuda(cudaMemcpyAsync(&h, w, sizeof h, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync")) return e;
    if (int e = check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return e;
    if (!h) return kSuccess;
    cudaMemsetAsync(w, 0, sizeof h, st);
    cudaStreamSynchronize(st);
    return set_error(kTimeout, "a staged kernel's wait for its bulk copies gave up");
}

int launch_blocks(const CompiledKernel& k, int threads, int64_t rows_per_block, int64_t rows) {
    const int sms = device_sms();
    const int per_sm = blocks_per_sm(k, threads);
    int64_t want = rows_per_block > 0 ? (rows + rows_per_block - 1) / rows_per_block : 1;
    int64_t cap = (int64_t)sms * per_sm;
    int64_t b = std::min<int64_t>(std::max<int64_t>(want, 1), cap);
    return (int)std::max<int64_t>(b, 1);
}

int perform_operation(gdf_column* const* outputs, int n_out, gdf_column* const* inputs, int n_in,
                      const ProgramArrays& pa, const EvalOptions& opt) {
    Program p;
    int rc = build_program(p, outputs, n_out, inputs, n_in, pa, opt.ignore_null_count);
    if (rc) return rc;
    const int64_t n = inputs[0]->size;
    if (n < 0) return set_error(kInvalidArgument, "negative row count");
    for (int c = 0; c < n_in; c++)
        if (inputs[c]->size < n) return set_error(kInvalidArgument, "input column shorter than input 0");
    for (int o = 0; o < n_out; o++)
        if (outputs[o]->size < n) return set_error(kInvalidArgument, "output column shorter than the input");

    Shape s = opt.shape.G > 0 ? opt.shape : eval_shape(p);
    // vector loads need every touched buffer aligned to G elements
    const auto ref = p.inputs_referenced();
    bool ok_align = true;
    for (int c = 0; c < n_in; c++) {
        if (ref[c] && n > 0 && !aligned(inputs[c]->data, (size_t)s.G * gdf_dtype_size(inputs[c]->dtype))) ok_align = false;
        if (inputs[c]->valid && !aligned(inputs[c]->valid, 4))
            return set_error(kInvalidArgument, "validity masks must be 4-byte aligned");
    }
    for (int o = 0; o < n_out; o++) {
        if (n > 0 && !aligned(outputs[o]->data, (size_t)s.G * gdf_dtype_size(outputs[o]->dtype))) ok_align = false;
        if (outputs[o]->valid && !aligned(outputs[o]->valid, 4))
            return set_error(kInvalidArgument, "validity masks must be 4-byte aligned");
    }
    if (!ok_align) { s.G = 1; s.J = 4; }
    // staged tiles: bulk copies need 16-byte aligned column and mask addresses
    if (s.tma_stages >= 2) {
        bool ok16 = ok_align && n > 0;
        for (int c = 0; c < n_in && ok16; c++)
            if ((ref[c] && !aligned(inputs[c]->data, 16)) || (inputs[c]->valid && !aligned(inputs[c]->valid, 16)))
                ok16 = false;
        if (!ok16 || eval_stage_bytes_per_warp(p, s) == 0) s.tma_stages = 0;
    }
    if (n > 0) {
        for (int c = 0; c < n_in; c++)
            if (ref[c] && !inputs[c]->data) return set_error(kInvalidArgument, "input column without data");
        for (int o = 0; o < n_out; o++)
            if (!outputs[o]->data) return set_error(kInvalidArgument, "output column without data");
    }

    const GeneratedKernel& gk = generated_eval(p, s);
    std::string err;
    const CompiledKernel* k = jit_get(gk, err);
    if (!k) return set_error(kJitError, err);
    const ParamLayout& L = k->layout;

    bool want_counts = opt.null_counts != nullptr;
    uint64_t* d_counts = nullptr;
    cudaStream_t st = opt.stream;
    if (want_counts) {
        if (int e = check_cuda(cudaMallocAsync((void**)&d_counts, sizeof(uint64_t) * n_out, st), "cudaMallocAsync"))
            return e;
        if (int e = check_cuda(cudaMemsetAsync(d_counts, 0, sizeof(uint64_t) * n_out, st), "cudaMemsetAsync"))
            return e;
    }
    std::vector<uint64_t> slots(L.total, 0);
    slots[L.n_rows] = (uint64_t)n;
    for (int c = 0; c < n_in; c++) {
        slots[L.in_data + c] = (uint64_t)(uintptr_t)inputs[c]->data;
        slots[L.in_valid + c] = (uint64_t)(uintptr_t)inputs[c]->valid;
    }
    for (int o = 0; o < n_out; o++) {
        slots[L.out_data + o] = (uint64_t)(uintptr_t)outputs[o]->data;
        slots[L.out_valid + o] = (uint64_t)(uintptr_t)outputs[o]->valid;
    }
    slots[L.counts] = (uint64_t)(uintptr_t)(d_counts ? d_counts : opt.device_valid_counts);
    const bool staged = k->dyn_smem > 0;
    if (staged) {
        unsigned long long* ew = device_error_word();
        if (!ew) return set_error(kAllocError, "device error word");
        slots[L.counts + 1] = (uint64_t)(uintptr_t)ew;
    }
    fill_scalars(p, L, slots);

    if (n > 0) {
        const int64_t rows_per_block = (int64_t)32 * s.G * s.J * (s.threads / 32);
        const int grid = launch_blocks(*k, s.threads, rows_per_block, n);
        void* args[] = {slots.data()};
        if (int e = check_cuda(cudaLaunchKernel((const void*)k->kernel, dim3(grid), dim3(s.threads), args,
                                                (size_t)k->dyn_smem, st),
                               "launch of the expression kernel"))
            return e;
        note_launch();
    }
    if (want_counts) {
        std::vector<uint64_t> h(n_out, 0);
        if (int e = check_cuda(cudaMemcpyAsync(h.data(), d_counts, sizeof(uint64_t) * n_out, cudaMemcpyDeviceToHost, st),
                               "cudaMemcpyAsync"))
            return e;
        cudaFreeAsync(d_counts, st);
        if (int e = check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return e;
        for (int o = 0; o < n_out; o++)
            opt.null_counts[o] = outputs[o]->valid ? (int64_t)n - (int64_t)h[o] : 0;
    } else if (opt.sync) {
        if (int e = check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize")) return e;
    }
    if (int e = check_cuda(cudaGetLastError(), "expression kernel")) return e;
    // a synchronous call with a staged kernel reports a wait that gave up (asynchronous calls leave
    // it to the next synchronous one on the device)
    if (staged && n > 0 && (want_counts || opt.sync))
        if (int e = take_device_error(st)) return e;
    return kSuccess;
}

namespace {

// Streams of the host-buffer path, per calling thread.
struct HostStreams {
    cudaStream_t s[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t ready = nullptr;
    ~HostStreams() {
        for (cudaStream_t& x : s)
            if (x) cudaStreamDestroy(x);
        if (ready) cudaEventDestroy(ready);
    }
};

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

int perform_operation_host(gdf_column* const* outputs, int n_out, gdf_column* const* inputs, int n_in,
                           const ProgramArrays& pa, int64_t chunk_rows) {
    if (!outputs || !inputs || n_out <= 0 || n_in <= 0) return set_error(kInvalidArgument, "null or empty column list");
    for (int c = 0; c < n_in; c++)
        if (!inputs[c]) return set_error(kInvalidArgument, "null input column");
    for (int o = 0; o < n_out; o++)
        if (!outputs[o]) return set_error(kInvalidArgument, "null output column");
    const int64_t n = inputs[0]->size;
    for (int c = 0; c < n_in; c++)
        if (inputs[c]->size != n) return set_error(kInvalidArgument, "input columns differ in size");
    for (int o = 0; o < n_out; o++)
        if (outputs[o]->size < n) return set_error(kInvalidArgument, "output column shorter than the input");
    {
        // the program is checked once up front (dtypes, registers, operators)
        Program p;
        if (int rc = build_program(p, outputs, n_out, inputs, n_in, pa, false)) return rc;
    }
    if (n == 0) {
        for (int o = 0; o < n_out; o++) outputs[o]->null_count = 0;
        return kSuccess;
    }
    // chunks start at multiples of 1024 rows: mask offsets are whole words and vector loads stay aligned
    int64_t chunk = chunk_rows > 0 ? chunk_rows : ((int64_t)4 << 20);
    chunk = std::max<int64_t>(1024, (chunk + 1023) / 1024 * 1024);
    if (chunk > n) chunk = (n + 1023) / 1024 * 1024;
    // streams belong to the device that was current when they were made: one set per device
    int dev = 0;
    if (check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return kCudaError;
    static thread_local std::map<int, HostStreams> per_device;
    HostStreams& hs = per_device[dev];
    for (cudaStream_t& x : hs.s)
        if (!x && check_cuda(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking), "cudaStreamCreate")) return kCudaError;
    if (!hs.ready && check_cuda(cudaEventCreateWithFlags(&hs.ready, cudaEventDisableTiming), "cudaEventCreate"))
        return kCudaError;
    // one device area per stream: every input and output column's chunk (data, then mask)
    auto mask_bytes = [](int64_t rows) { return round256((size_t)gdf_valid_allocation_size(rows)); };
    size_t per_slot = 0;
    for (int c = 0; c < n_in; c++)
        per_slot += round256((size_t)chunk * gdf_dtype_size(inputs[c]->dtype)) + (inputs[c]->valid ? mask_bytes(chunk) : 0);
    for (int o = 0; o < n_out; o++)
        per_slot += round256((size_t)chunk * gdf_dtype_size(outputs[o]->dtype)) + (outputs[o]->valid ? mask_bytes(chunk) : 0);
    char* area[3] = {nullptr, nullptr, nullptr};
    uint64_t* d_counts = nullptr;
    int rc = kSuccess;
    auto release = [&]() {
        for (int k = 0; k < 3; k++) {
            cudaStreamSynchronize(hs.s[k]);
            if (area[k]) cudaFreeAsync(area[k], hs.s[k]);
        }
        if (d_counts) cudaFreeAsync(d_counts, hs.s[0]);
        cudaStreamSynchronize(hs.s[0]);
    };
    if ((rc = check_cuda(cudaMallocAsync((void**)&d_counts, sizeof(uint64_t) * n_out, hs.s[0]), "cudaMallocAsync")) ||
        (rc = check_cuda(cudaMemsetAsync(d_counts, 0, sizeof(uint64_t) * n_out, hs.s[0]), "cudaMemsetAsync"))) {
        release();
        return rc;
    }
    cudaEventRecord(hs.ready, hs.s[0]);
    for (int k = 0; k < 3; k++) {
        if ((rc = check_cuda(cudaMallocAsync((void**)&area[k], per_slot, hs.s[k]), "cudaMallocAsync"))) {
            release();
            return rc;
        }
        cudaStreamWaitEvent(hs.s[k], hs.ready, 0);
    }
    std::vector<gdf_column> vin(n_in), vout(n_out);
    std::vector<gdf_column*> pin(n_in), pout(n_out);
    const int64_t nchunks = (n + chunk - 1) / chunk;
    for (int64_t q = 0; q < nchunks && rc == kSuccess; q++) {
        const int k = (int)(q % 3);
        cudaStream_t st = hs.s[k];
        const int64_t off = q * chunk;
        const int64_t r = std::min(chunk, n - off);
        const size_t mb = (size_t)((r + 7) / 8);
        char* cur = area[k];
        for (int c = 0; c < n_in; c++) {
            const size_t w = gdf_dtype_size(inputs[c]->dtype);
            vin[c] = *inputs[c];
            vin[c].size = (gdf_size_type)r;
            vin[c].data = cur;
            cudaMemcpyAsync(cur, (const char*)inputs[c]->data + off * w, (size_t)r * w, cudaMemcpyHostToDevice, st);
            cur += round256((size_t)chunk * w);
            if (inputs[c]->valid) {
                vin[c].valid = (gdf_valid_type*)cur;
                cudaMemcpyAsync(cur, (const char*)inputs[c]->valid + off / 8, mb, cudaMemcpyHostToDevice, st);
                cur += mask_bytes(chunk);
            }
            pin[c] = &vin[c];
        }
        for (int o = 0; o < n_out; o++) {
            const size_t w = gdf_dtype_size(outputs[o]->dtype);
            vout[o] = *outputs[o];
            vout[o].size = (gdf_size_type)r;
            vout[o].data = cur;
            cur += round256((size_t)chunk * w);
            if (outputs[o]->valid) {
                vout[o].valid = (gdf_valid_type*)cur;
                cur += mask_bytes(chunk);
            }
            pout[o] = &vout[o];
        }
        EvalOptions eo;
        eo.stream = st;
        eo.sync = false;
        eo.device_valid_counts = d_counts;
        if ((rc = perform_operation(pout.data(), n_out, pin.data(), n_in, pa, eo))) break;
        for (int o = 0; o < n_out; o++) {
            const size_t w = gdf_dtype_size(outputs[o]->dtype);
            cudaMemcpyAsync((char*)outputs[o]->data + off * w, vout[o].data, (size_t)r * w, cudaMemcpyDeviceToHost, st);
            if (outputs[o]->valid)
                cudaMemcpyAsync((char*)outputs[o]->valid + off / 8, vout[o].valid, mb, cudaMemcpyDeviceToHost, st);
        }
    }
    if (rc == kSuccess) {
        for (int k = 1; k < 3; k++) {
            cudaEventRecord(hs.ready, hs.s[k]);
            cudaStreamWaitEvent(hs.s[0], hs.ready, 0);
        }
        std::vector<uint64_t> h(n_out, 0);
        cudaMemcpyAsync(h.data(), d_counts, sizeof(uint64_t) * n_out, cudaMemcpyDeviceToHost, hs.s[0]);
        if (!(rc = check_cuda(cudaStreamSynchronize(hs.s[0]), "host-buffer evaluation")))
            for (int o = 0; o < n_out; o++) outputs[o]->null_count = outputs[o]->valid ? (gdf_size_type)(n - (int64_t)h[o]) : 0;
    }
    release();
    if (rc == kSuccess) rc = check_cuda(cudaGetLastError(), "host-buffer evaluation");
    return rc;
}

}  // namespace ral
