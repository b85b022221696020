// batch.h — many register programs in one persistent launch, replayed as a CUDA graph.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "codegen.h"
#include "engine.h"
#include "jit.h"
#include "program.h"

namespace ral {

struct BatchEntry {
    Program program;
    std::vector<gdf_column> inputs, outputs;  // copies of the caller's column descriptors
    Shape shape;
    int64_t rows = 0;
    int64_t items = 0;  // warp tiles
};

class Batch {
public:
    ~Batch();
    // Adds one program (perform_operation arguments); returns its index or a negative status.
    int add(gdf_column* const* outputs, int n_out, gdf_column* const* inputs, int n_in, const ProgramArrays& pa);
    // Chooses shapes, compiles the batch kernel, uploads descriptors, captures the graph.
    int prepare(cudaStream_t stream);
    // Runs every program once (graph replay when use_graph).
    int run(cudaStream_t stream, bool use_graph);
    int programs() const { return (int)entries_.size(); }
    int64_t total_rows() const;
    int64_t total_items() const { return total_items_; }
    const std::string& kernel_name() const { return kernel_name_; }
    int registers() const { return registers_; }
    int grid() const { return grid_; }
    int blocks_per_sm() const { return per_sm_; }
    // Generated source (and an NVRTC-only compile) for the programs added so far.
    int debug_source(bool compile, std::string& source, std::string& log) const;
    // Every program of the batch at this tile shape instead of the tuned one (autotuning).
    void force_shape(int J, int U, bool soft) { forced_J_ = J; forced_U_ = U; forced_S_ = soft; }

private:
    int launch(cudaStream_t stream);
    std::vector<std::unique_ptr<BatchEntry>> entries_;
    std::string kernel_name_;
    const CompiledKernel* kernel_ = nullptr;
    int stride_ = 1;
    size_t smem_ = 0;
    void* d_descs_ = nullptr;
    void* d_prefix_ = nullptr;
    void* d_fn_ = nullptr;
    unsigned int* d_counter_ = nullptr;
    int64_t total_items_ = 0;
    int grid_ = 0;
    int per_sm_ = 0;
    int registers_ = 0;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    bool prepared_ = false;
    int forced_J_ = 0, forced_U_ = 1;
    bool forced_S_ = false;
};

// Tile shape of a program's batch item: slices per warp tile J, the unroll of the slice loop and
// whether its double operations run on the integer pipes, from the autotuner's table (keyed by
// dtype mix and program length) or the default (J = 8 / G, no unroll, FP64 instructions).
Shape tuned_shape(const Program& p, int G);
// Records a measured best for the program's key in the autotuner's table (persisted as JSON
// in the JIT cache directory).
void record_tuned_shape(const Program& p, int G, int J, int U, bool soft, double ms);
std::string tune_key(const Program& p, int G);

// Consecutive work items a batch warp takes per atomic (RAL_BATCH_GRAB, default 1).
int batch_grab();

// Compiles generated relocatable TUs on a pool of host threads (cached per name); appends the
// ptxas logs to *logs when given.
int compile_items(const std::vector<GeneratedKernel>& items, std::vector<const std::vector<char>*>& objects,
                  std::string* logs);

}  // namespace ral
