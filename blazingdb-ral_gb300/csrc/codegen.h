// codegen.h — CUDA source generation for one register program.
//
// The reference interprets the program per row with a shared-memory register
// file and a three-level type dispatch per op (src/Interpreter/
// interpreter_ops.cuh:473-838, 1417-1458).  Here each program becomes its own
// kernel: registers are SSA values in thread registers, every op is a single
// typed expression, each input column is read once with vector loads and
// validity is computed 32 rows per 32-bit word in the same pass.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "program.h"

namespace ral {

// Launch shape of a generated kernel.
struct Shape {
    int G = 2;         // consecutive rows per lane per slice (a vector load covers G elements)
    int J = 2;         // slices per warp tile
    int threads = 256; // threads per block
    int min_blocks = 1;  // __launch_bounds__ minimum resident blocks per SM
};

// Slot order of the kernel's parameter block (all 8-byte slots).
struct ParamLayout {
    int n_rows = 0;
    int in_data = 0, in_valid = 0;      // first slot of n_in pointers each
    int out_data = 0, out_valid = 0;    // first slot of n_out pointers each
    int counts = 0;                     // device array: per output, count of valid bits
    int scratch = -1;                   // filter kernels: scratch block
    int capacity = -1;                  // filter kernels: output capacity in rows
    int gather_data = -1, gather_valid = -1, gather_out = -1, gather_out_valid = -1;  // filter kernels
    std::vector<int> lscalar_slot, rscalar_slot;  // per op, -1 if none
    int total = 0;
};

// Largest element width (bytes) over the columns a kernel reads or writes.
int max_width(const Program& p);
// Default shape for a program: G = 16 / widest column, J so that a lane covers 4 rows.
Shape default_shape(const Program& p);

struct GeneratedKernel {
    std::string name;
    std::string source;   // full translation unit (prelude prepended by the JIT)
    ParamLayout layout;
    Shape shape;
};

// perform_operation: evaluate the program over n rows into the outputs.
GeneratedKernel generate_eval_kernel(const Program& p, const Shape& s);

// Filter description for the fused stencil/compaction/gather kernel.
struct FilterSpec {
    // predicate: either a program with one INT8 output (the stencil), or a
    // clone of a one-byte frame column (evaluate_expression's "$n" shortcut)
    bool clone_stencil = false;
    int clone_column = -1;            // frame column index when clone_stencil
    bool clone_has_valid = false;
    const Program* predicate = nullptr;   // inputs are frame columns predicate_cols[i]
    std::vector<int> predicate_cols;
    // gathered columns (every frame column, in order)
    std::vector<gdf_dtype> gather_dtypes;
    std::vector<bool> gather_has_valid;
    std::vector<int> gather_frame_col;    // frame column index of each gathered column
    int n_frame = 0;
};

GeneratedKernel generate_filter_kernel(const FilterSpec& f, const Shape& s);

// C type name of a column element.
const char* element_ctype(gdf_dtype t);

}  // namespace ral
