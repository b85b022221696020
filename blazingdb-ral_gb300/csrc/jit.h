// jit.h — NVRTC compilation and caching of generated kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "codegen.h"

namespace ral {

struct CompiledKernel {
    cudaLibrary_t library = nullptr;
    cudaKernel_t kernel = nullptr;
    std::string name;
    ParamLayout layout;
    Shape shape;
    int dyn_smem = 0;             // dynamic shared memory per block (staged eval kernels)
    size_t cubin_bytes = 0;
    double compile_ms = 0.0;      // 0 when it came from the disk cache
    std::string ptxas_log;
};

// Compiles (or fetches from cache) the kernel; thread-safe.  The returned
// pointer stays valid for the life of the process.  Returns nullptr and sets
// err on failure.
const CompiledKernel* jit_get(const GeneratedKernel& gk, std::string& err);

// Compiles to a cubin without loading it (no GPU needed).  Returns false and
// sets err on failure; fills cubin size and the ptxas -v log.
bool jit_compile_only(const GeneratedKernel& gk, size_t* cubin_bytes, std::string* ptxas_log, std::string& err);

// Relocatable device code (-rdc) of one generated TU, compiled to a cubin object; cached in
// memory and on disk by name and source hash.  Thread-safe; compiles of different TUs run
// concurrently.  Returns nullptr and sets err on failure.
const std::vector<char>* jit_object(const GeneratedKernel& gk, std::string& err, std::string* ptxas_log = nullptr);

// Links relocatable objects with nvJitLink, loads the image and returns its kernel `kernel_name`;
// cached in memory by `key`.  Returns nullptr and sets err on failure.
const CompiledKernel* jit_link(const std::string& key, const std::string& kernel_name,
                               const std::vector<const std::vector<char>*>& objects, std::string& err);

// The same link without loading (no GPU needed); fills the linked size and the link log.
bool jit_link_only(const std::vector<const std::vector<char>*>& objects, size_t* bytes, std::string* log,
                   std::string& err);

struct JitStats {
    long long compiles = 0;
    long long disk_hits = 0;
    long long memory_hits = 0;
    double compile_ms_total = 0.0;
};
JitStats jit_stats();

// The device prelude (device_rt.cuh), embedded at build time.
const char* jit_prelude();

}  // namespace ral
