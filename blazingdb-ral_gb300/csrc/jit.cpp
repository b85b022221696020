// jit.cpp — NVRTC compilation and caching of generated kernels.
//
// Kernels are compiled for sm_103a with --fmad=false (no multiply-add
// contraction, so double results match the reference's separately rounded
// C++ operations) and cached twice: in memory by kernel name, and as cubin
// files on disk (RAL_JIT_CACHE_DIR, default $HOME/.cache/ralgpu-jit) keyed by
// a hash of the full source and the NVRTC version.
#include "jit.h"

#include <nvJitLink.h>
#include <nvrtc.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <mutex>
#include <sstream>
#include <sys/stat.h>
#include <unistd.h>
#include <unordered_map>
#include <vector>

extern "C" const char* const ral_prelude_source;

namespace ral {

const char* jit_prelude() { return ral_prelude_source; }

namespace {

std::mutex g_mu;
std::unordered_map<std::string, std::unique_ptr<CompiledKernel>> g_cache;
JitStats g_stats;

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull) {
    for (unsigned char c : s) { h ^= c; h *= 1099511628211ull; }
    return h;
}

// RAL_SOFT_FP=0 selects the hardware FP64 instructions for the operations that otherwise run
// on the integer pipes (same results; for comparison and diagnosis); kernels whose
// GeneratedKernel::soft_fp is false always use them
const std::string& trig_define() {
    // RAL_SOFT_TRIG=1: the integer-pipe sin / cos in every kernel (the same choice everywhere,
    // since the two differ in the last bit)
    static const std::string d = [] {
        const char* e = std::getenv("RAL_SOFT_TRIG");
        return std::string("#define RAL_SOFT_TRIG ") + ((e && std::string(e) == "1") ? "1" : "0") + "\n";
    }();
    return d;
}

const std::string& soft_fp_define(bool soft) {
    static const std::string off = "#define RAL_SOFT_FP 0\n";
    if (!soft) return off;
    static const std::string d = [] {
        const char* e = std::getenv("RAL_SOFT_FP");
        std::string out = std::string("#define RAL_SOFT_FP ") + ((e && std::string(e) == "0") ? "0" : "1") + "\n";
        // RAL_SOFT_INT_DIV=0|1|2|3: the compiler's 64-bit division / integer-only division for
        // every divisor / for 32-bit divisors / for divisors below 2^16 (the default)
        const char* i = std::getenv("RAL_SOFT_INT_DIV");
        if (i && (std::string(i) == "0" || std::string(i) == "1" || std::string(i) == "2" || std::string(i) == "3"))
            out += std::string("#define RAL_SOFT_INT_DIV ") + i + "\n";
        // RAL_SOFT_ROUND=0: floor / ceil on the FP64 pipe
        const char* r = std::getenv("RAL_SOFT_ROUND");
        if (r && std::string(r) == "0") out += "#define RAL_SOFT_ROUND 0\n";
        return out;
    }();
    return d;
}

std::string full_source(const GeneratedKernel& gk) {
    return trig_define() + soft_fp_define(gk.soft_fp) + std::string(ral_prelude_source) + "\n" + gk.source;
}

std::string cache_dir() {
    const char* d = std::getenv("RAL_JIT_CACHE_DIR");
    if (d && *d) return d;
    const char* home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/ralgpu-jit";
}

void mkdirs(const std::string& path) {
    std::string cur;
    std::stringstream ss(path);
    std::string part;
    if (!path.empty() && path[0] == '/') cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty()) continue;
        cur += part + "/";
        mkdir(cur.c_str(), 0755);
    }
}

std::string disk_key(const GeneratedKernel& gk) {
    int major = 0, minor = 0;
    nvrtcVersion(&major, &minor);
    char buf[96];
    snprintf(buf, sizeof buf, "%s_%016llx_nvrtc%d.%d_sm103a.cubin", gk.name.c_str(),
             (unsigned long long)fnv1a(full_source(gk)), major, minor);
    return buf;
}

// Register cap of relocatable item functions (RAL_BATCH_MAXRREG).  Default 80 (three blocks of
// 256 threads per SM): on the 256-program mix 80 / 96 / 64 ran 116.2 / 118.2 / 116.9 ms and, over
// tables capped at 1M rows, 80 / 96 ran 14.12 / 14.30 ms.
int relocatable_max_registers() {
    const char* e = std::getenv("RAL_BATCH_MAXRREG");
    const int v = e && *e ? std::atoi(e) : 80;
    return v >= 32 && v <= 255 ? v : 80;
}

bool compile(const GeneratedKernel& gk, std::vector<char>& cubin, std::string& log, std::string& err,
             bool relocatable = false) {
    const std::string src = full_source(gk);
    nvrtcProgram prog;
    nvrtcResult rc = nvrtcCreateProgram(&prog, src.c_str(), (gk.name + ".cu").c_str(), 0, nullptr, nullptr);
    if (rc != NVRTC_SUCCESS) { err = std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(rc); return false; }
    std::vector<const char*> opts = {"--gpu-architecture=sm_103a", "--fmad=false", "--std=c++17", "-lineinfo",
                                     "--ptxas-options=-v"};
    std::string maxreg;
    if (relocatable) {
        opts.push_back("--relocatable-device-code=true");
        // item functions are compiled apart from the kernel that calls them, so launch bounds do
        // not reach them: cap their registers so the linked kernel keeps its occupancy
        maxreg = "--maxrregcount=" + std::to_string(gk.max_registers > 0 ? gk.max_registers : relocatable_max_registers());
        opts.push_back(maxreg.c_str());
    }
    rc = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
    size_t log_size = 0;
    nvrtcGetProgramLogSize(prog, &log_size);
    log.assign(log_size, '\0');
    if (log_size) nvrtcGetProgramLog(prog, &log[0]);
    while (!log.empty() && log.back() == '\0') log.pop_back();
    if (rc != NVRTC_SUCCESS) {
        err = std::string("NVRTC compile of ") + gk.name + " failed: " + nvrtcGetErrorString(rc) + "\n" + log;
        nvrtcDestroyProgram(&prog);
        return false;
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    cubin.resize(n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    return true;
}

}  // namespace

bool jit_compile_only(const GeneratedKernel& gk, size_t* cubin_bytes, std::string* ptxas_log, std::string& err) {
    std::vector<char> cubin;
    std::string log;
    if (!compile(gk, cubin, log, err)) return false;
    if (cubin_bytes) *cubin_bytes = cubin.size();
    if (ptxas_log) *ptxas_log = log;
    return true;
}

const CompiledKernel* jit_get(const GeneratedKernel& gk, std::string& err) {
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_cache.find(gk.name);
        if (it != g_cache.end()) {
            g_stats.memory_hits++;
            return it->second.get();
        }
    }
    // compile (or read the disk cache) outside the lock, so different kernels compile concurrently
    std::vector<char> cubin;
    std::string log;
    double ms = 0.0;
    const std::string dir = cache_dir();
    const std::string path = dir + "/" + disk_key(gk);
    bool from_disk = false;
    {
        std::ifstream f(path, std::ios::binary);
        if (f) {
            cubin.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
            from_disk = !cubin.empty();
        }
    }
    if (!from_disk) {
        auto t0 = std::chrono::steady_clock::now();
        if (!compile(gk, cubin, log, err)) return nullptr;
        ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        mkdirs(dir);
        const std::string tmp = path + ".tmp" + std::to_string(getpid()) + "_" +
                                std::to_string((unsigned long long)(uintptr_t)cubin.data());
        std::ofstream f(tmp, std::ios::binary);
        if (f) {
            f.write(cubin.data(), (std::streamsize)cubin.size());
            f.close();
            std::rename(tmp.c_str(), path.c_str());
        }
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (from_disk) g_stats.disk_hits++;
    else {
        g_stats.compiles++;
        g_stats.compile_ms_total += ms;
    }
    auto it = g_cache.find(gk.name);
    if (it != g_cache.end()) return it->second.get();  // another thread finished first
    auto ck = std::make_unique<CompiledKernel>();
    cudaError_t ce = cudaLibraryLoadData(&ck->library, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (ce != cudaSuccess) {
        err = std::string("cudaLibraryLoadData(") + gk.name + "): " + cudaGetErrorString(ce);
        cudaGetLastError();
        return nullptr;
    }
    ce = cudaLibraryGetKernel(&ck->kernel, ck->library, gk.name.c_str());
    if (ce != cudaSuccess) {
        err = std::string("cudaLibraryGetKernel(") + gk.name + "): " + cudaGetErrorString(ce);
        cudaGetLastError();
        return nullptr;
    }
    ck->name = gk.name;
    ck->layout = gk.layout;
    ck->shape = gk.shape;
    ck->dyn_smem = gk.dyn_smem;
    if (gk.dyn_smem > 48 * 1024) {
        ce = cudaFuncSetAttribute((const void*)ck->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, gk.dyn_smem);
        if (ce != cudaSuccess) {
            err = std::string("cudaFuncSetAttribute(") + gk.name + "): " + cudaGetErrorString(ce);
            return nullptr;
        }
    }
    ck->cubin_bytes = cubin.size();
    ck->compile_ms = ms;
    ck->ptxas_log = log;
    const CompiledKernel* out = ck.get();
    g_cache.emplace(gk.name, std::move(ck));
    return out;
}

namespace {

std::mutex g_obj_mu;
std::unordered_map<std::string, std::unique_ptr<std::vector<char>>> g_objects;
std::unordered_map<std::string, std::unique_ptr<CompiledKernel>> g_linked;

bool link_objects(const std::vector<const std::vector<char>*>& objects, std::vector<char>& image, std::string& log,
                  std::string& err) {
    nvJitLinkHandle h;
    const char* opts[] = {"-arch=sm_103a"};
    nvJitLinkResult rc = nvJitLinkCreate(&h, 1, opts);
    if (rc != NVJITLINK_SUCCESS) { err = "nvJitLinkCreate failed (" + std::to_string((int)rc) + ")"; return false; }
    for (size_t i = 0; i < objects.size() && rc == NVJITLINK_SUCCESS; i++) {
        const std::string nm = "obj" + std::to_string(i) + ".cubin";
        rc = nvJitLinkAddData(h, NVJITLINK_INPUT_CUBIN, objects[i]->data(), objects[i]->size(), nm.c_str());
    }
    if (rc == NVJITLINK_SUCCESS) rc = nvJitLinkComplete(h);
    size_t n = 0;
    if (nvJitLinkGetInfoLogSize(h, &n) == NVJITLINK_SUCCESS && n > 1) {
        std::string info(n, '\0');
        nvJitLinkGetInfoLog(h, &info[0]);
        while (!info.empty() && info.back() == '\0') info.pop_back();
        log += info;
    }
    if (rc != NVJITLINK_SUCCESS) {
        std::string elog;
        if (nvJitLinkGetErrorLogSize(h, &n) == NVJITLINK_SUCCESS && n > 1) {
            elog.assign(n, '\0');
            nvJitLinkGetErrorLog(h, &elog[0]);
            while (!elog.empty() && elog.back() == '\0') elog.pop_back();
        }
        err = "nvJitLink failed (" + std::to_string((int)rc) + "): " + elog;
        nvJitLinkDestroy(&h);
        return false;
    }
    nvJitLinkGetLinkedCubinSize(h, &n);
    image.resize(n);
    nvJitLinkGetLinkedCubin(h, image.data());
    nvJitLinkDestroy(&h);
    return true;
}

}  // namespace

const std::vector<char>* jit_object(const GeneratedKernel& gk, std::string& err, std::string* ptxas_log) {
    {
        std::lock_guard<std::mutex> lock(g_obj_mu);
        auto it = g_objects.find(gk.name);
        if (it != g_objects.end()) {
            std::lock_guard<std::mutex> l2(g_mu);
            g_stats.memory_hits++;
            return it->second.get();
        }
    }
    auto obj = std::make_unique<std::vector<char>>();
    const std::string dir = cache_dir();
    const std::string path = dir + "/" + disk_key(gk) + ".r" +
                             std::to_string(gk.max_registers > 0 ? gk.max_registers : relocatable_max_registers()) + ".rdc";
    bool from_disk = false;
    {
        std::ifstream f(path, std::ios::binary);
        if (f) {
            obj->assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
            from_disk = !obj->empty();
        }
    }
    if (!from_disk) {
        std::string log;
        auto t0 = std::chrono::steady_clock::now();
        if (!compile(gk, *obj, log, err, true)) return nullptr;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (ptxas_log) *ptxas_log = log;
        {
            std::lock_guard<std::mutex> l2(g_mu);
            g_stats.compiles++;
            g_stats.compile_ms_total += ms;
        }
        mkdirs(dir);
        const std::string tmp = path + ".tmp" + std::to_string(getpid()) + "_" +
                                std::to_string((unsigned long long)(uintptr_t)obj.get());
        std::ofstream f(tmp, std::ios::binary);
        if (f) {
            f.write(obj->data(), (std::streamsize)obj->size());
            f.close();
            std::rename(tmp.c_str(), path.c_str());
        }
    } else {
        std::lock_guard<std::mutex> l2(g_mu);
        g_stats.disk_hits++;
    }
    std::lock_guard<std::mutex> lock(g_obj_mu);
    auto ins = g_objects.emplace(gk.name, std::move(obj));
    return ins.first->second.get();
}

bool jit_link_only(const std::vector<const std::vector<char>*>& objects, size_t* bytes, std::string* log,
                   std::string& err) {
    std::vector<char> image;
    std::string l;
    if (!link_objects(objects, image, l, err)) return false;
    if (bytes) *bytes = image.size();
    if (log) *log = l;
    return true;
}

const CompiledKernel* jit_link(const std::string& key, const std::string& kernel_name,
                               const std::vector<const std::vector<char>*>& objects, std::string& err) {
    std::lock_guard<std::mutex> lock(g_obj_mu);
    auto it = g_linked.find(key);
    if (it != g_linked.end()) return it->second.get();
    std::vector<char> image;
    std::string log;
    auto t0 = std::chrono::steady_clock::now();
    if (!link_objects(objects, image, log, err)) return nullptr;
    auto ck = std::make_unique<CompiledKernel>();
    cudaError_t ce = cudaLibraryLoadData(&ck->library, image.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (ce != cudaSuccess) {
        err = std::string("cudaLibraryLoadData(") + kernel_name + "): " + cudaGetErrorString(ce);
        cudaGetLastError();
        return nullptr;
    }
    ce = cudaLibraryGetKernel(&ck->kernel, ck->library, kernel_name.c_str());
    if (ce != cudaSuccess) {
        err = std::string("cudaLibraryGetKernel(") + kernel_name + "): " + cudaGetErrorString(ce);
        cudaGetLastError();
        return nullptr;
    }
    ck->name = kernel_name;
    ck->cubin_bytes = image.size();
    ck->compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    ck->ptxas_log = log;
    const CompiledKernel* out = ck.get();
    g_linked.emplace(key, std::move(ck));
    return out;
}

JitStats jit_stats() {
    std::lock_guard<std::mutex> lock(g_mu);
    return g_stats;
}

}  // namespace ral
