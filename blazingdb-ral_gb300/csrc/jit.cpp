// jit.cpp — NVRTC compilation and caching of generated kernels.
//
// Kernels are compiled for sm_103a with --fmad=false (no multiply-add
// contraction, so double results match the reference's separately rounded
// C++ operations) and cached twice: in memory by kernel name, and as cubin
// files on disk (RAL_JIT_CACHE_DIR, default $HOME/.cache/ralgpu-jit) keyed by
// a hash of the full source and the NVRTC version.
#include "jit.h"

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

std::string full_source(const GeneratedKernel& gk) {
    return std::string(ral_prelude_source) + "\n" + gk.source;
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

bool compile(const GeneratedKernel& gk, std::vector<char>& cubin, std::string& log, std::string& err) {
    const std::string src = full_source(gk);
    nvrtcProgram prog;
    nvrtcResult rc = nvrtcCreateProgram(&prog, src.c_str(), (gk.name + ".cu").c_str(), 0, nullptr, nullptr);
    if (rc != NVRTC_SUCCESS) { err = std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(rc); return false; }
    const char* opts[] = {"--gpu-architecture=sm_103a", "--fmad=false", "--std=c++17", "-lineinfo",
                          "--ptxas-options=-v"};
    rc = nvrtcCompileProgram(prog, (int)(sizeof opts / sizeof opts[0]), opts);
    size_t log_size = 0;
    nvrtcGetProgramLogSize(prog, &log_size);
    log.assign(log_size, '\0');
    if (log_size) nvrtcGetProgramLog(prog, &log[0]);
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
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(gk.name);
    if (it != g_cache.end()) {
        g_stats.memory_hits++;
        return it->second.get();
    }
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
        g_stats.compiles++;
        g_stats.compile_ms_total += ms;
        mkdirs(dir);
        const std::string tmp = path + ".tmp" + std::to_string(getpid());
        std::ofstream f(tmp, std::ios::binary);
        if (f) {
            f.write(cubin.data(), (std::streamsize)cubin.size());
            f.close();
            std::rename(tmp.c_str(), path.c_str());
        }
    } else {
        g_stats.disk_hits++;
    }
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
    ck->cubin_bytes = cubin.size();
    ck->compile_ms = ms;
    ck->ptxas_log = log;
    const CompiledKernel* out = ck.get();
    g_cache.emplace(gk.name, std::move(ck));
    return out;
}

JitStats jit_stats() {
    std::lock_guard<std::mutex> lock(g_mu);
    return g_stats;
}

}  // namespace ral
