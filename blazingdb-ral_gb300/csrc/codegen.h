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
    int unroll = 4;    // filter kernels: unroll of the predicate pass over slices
    bool stage = false;  // filter kernels: dense slices written through a shared-memory stage
    bool soft = false;   // batch items: integer-pipe double operations (the autotuner decides)
    // filter kernels: slices of pass 2 prefetched into L2 ahead (0, the default: none -- measured
    // slower at 4, 8 and 16 slices: 500M rows at s = 0.5 ran 5.39 / 5.71 / 5.79 ms against 5.06).
    // With the dense pass 2 any value > 0 prefetches the chunk's columns during the look-back
    // (also slower: the 200M-row filter + project at s = 0.5 ran 2.53 ms against 2.09).
    int prefetch = 0;
    // eval kernels: 0 loads every tile from global memory into registers; S >= 2 stages each warp's
    // tiles in shared memory through a ring of S stages filled by bulk copies (TMA), the next
    // tiles in flight while the warp computes the current one
    int tma_stages = 0;
    // filter kernels: pass 2 walks a shared-memory list of the chunk's kept rows, 32 at a time,
    // so every lane evaluates or gathers a kept row and stores are contiguous (1, the default;
    // -1 is the same), or takes its own G rows of each slice, skipping dropped ones (0)
    int dense = -1;
    // dense pass 2: list steps whose loads are issued together (1 or 2; 2 measured no faster:
    // 2.15 ms against 2.09 at s = 0.5, at five blocks per SM for its registers)
    int dense_unroll = 1;
    // filter kernels: 0 (default) takes chunks by ticket and finds each chunk's output offset by
    // look-back; K > 0 gives each warp K consecutive chunks of a cooperative launch and one
    // grid-wide barrier between pass 1 and pass 2 (the offsets are then sums of block, warp and
    // chunk counts), for launches small enough that every block is resident
    int grid_k = 0;
};

// Slot order of the kernel's parameter block (all 8-byte slots).
struct ParamLayout {
    int n_rows = 0;
    int in_data = 0, in_valid = 0;      // first slot of the input (eval) or frame (filter) pointers
    int out_data = 0, out_valid = 0;    // first slot of the output pointers
    int counts = -1;                    // eval kernels: per output, count of valid bits
    int scratch = -1;                   // filter kernels: scratch block
    // filter kernels: output row offset, 0 .. 31 -- kept row j is written at row obase + j of the
    // output pointers and bit obase + j of the output masks (a chunk appended into a mask word
    // that earlier rows have started); -1 in item functions
    int obase = -1;
    // filter kernels with Shape::grid_k: the grid counter's value before the launch, and the
    // device address of the caller's host-mapped header (the last block to finish writes the
    // header there, then a completion tag)
    int epoch = -1;
    int hostmap = -1;
    std::vector<int> lscalar_slot, rscalar_slot;  // per op of the (predicate) program, -1 if none
    // per op: for an integer division or remainder by a literal, the first of two slots holding
    // the literal's precomputed multiplier and shift (ral_sf_make_divider), -1 if none
    std::vector<int> rdiv_slot;
    int total = 0;
};

// True for an integer division or remainder whose divisor is a literal (computed with a
// multiplier precomputed on the host instead of a division per row).
bool divides_by_int_literal(const Op& op);
// Gives each literal operand of p's ops its slot (and an integer divisor its two divider slots),
// from `slot` on.
void assign_scalar_slots(const Program& p, ParamLayout& L, int& slot);

// Largest element width (bytes) over the columns a kernel reads or writes.
int max_width(const Program& p);
// Default shape for a program: G = 16 / widest column, J so that a lane covers 4 rows.
Shape default_shape(const Program& p);
// Applies "J=8,U=2,T=128,B=3,S=1,P=8" style overrides (slices, unroll, threads, min blocks per
// SM, staging, L2 prefetch distance) to a shape; unknown keys and out-of-range values are ignored.
void apply_shape_tune(Shape& sh, const std::string& t);

struct GeneratedKernel {
    std::string name;
    std::string source;   // full translation unit (prelude prepended by the JIT)
    ParamLayout layout;
    Shape shape;
    // filter kernels: scalar slots of the projection program
    std::vector<int> layout_project_lscalar, layout_project_rscalar;
    std::vector<int> layout_project_rdiv;
    // filter item functions: shared-memory words the function needs in its warp's area
    int item_smem_words = 0;
    // integer-pipe double operations (softfp.cuh) unless RAL_SOFT_FP=0.  Batched item functions
    // take it from their shape (the autotuner's choice; by default the FP64 instructions, since
    // under the items' register cap the larger integer-pipe code spills: 256 programs over tables
    // capped at 1M rows ran 31.6 ms with it against 20.4 ms without).
    bool soft_fp = true;
    // relocatable item functions: register cap (0: RAL_BATCH_MAXRREG's)
    int max_registers = 0;
    // dynamic shared memory a block needs (staged eval kernels)
    int dyn_smem = 0;
};

// Shared-memory bytes one warp of a staged eval kernel needs (its barriers and S stages), or 0
// when the program cannot be staged (a tile of a column not a multiple of 16 bytes).
int eval_stage_bytes_per_warp(const Program& p, const Shape& s);

// Batched and served launches run many programs in one persistent kernel.  Each program's warp
// tile is a relocatable device function of its own, compiled once per program structure and
// shape and cached:
//   extern "C" __device__ void <name>(const ral_u64* slots, long long tile)
// with slots laid out as gk.layout.  A dispatcher kernel, linked with the item functions, takes
// work items (program, tile) from a device counter in chunks, finds the program by binary search
// over the item prefix (in shared memory) and calls its function:
//   <name>(const ral_u64* descs, int stride, const long long* item_prefix, const long long* item_base,
//          const int* fn_index, int n_programs, unsigned int* counter, long long total_items)
// descs holds `stride` slots per program; fn_index[q] indexes the item functions; item t of
// program q runs tile item_base[q] + t (item_base may be null: all 0), so a request's chunks can
// be spread over several launches.  Items run in program order: interleaving the programs' tiles
// (tried: every program's tiles spread evenly over the sequence) made the 256-program batch 14x
// slower, each warp's consecutive items then touching different code and different tables.
// Filter + project requests are batched the same way: their item function is the fused filter
// kernel's chunk body (generate_filter_kernel with item = true),
//   extern "C" __device__ void <name>(const ral_u64* slots, long long chunk, unsigned* warp_smem)
// which also takes the calling warp's area of the dispatcher's dynamic shared memory.
GeneratedKernel generate_batch_item(const Program& p, const Shape& s);
struct DispatchEntry {
    std::string name;
    bool filter = false;  // takes the warp's shared-memory area
};
// smem_words_per_warp: largest item_smem_words over the filter items (0 if none).  The dynamic
// shared memory is then (n_programs + 1) * 8 + n_programs * 12 (rounded up to 16) plus
// 8 warps * smem_words_per_warp * 4 bytes.  A warp takes `grab` consecutive items per atomic
// and runs them in order.  Filter items need grab = 1: a chunk's look-back waits on the chunk
// before it, so a warp holding several consecutive chunks would make the next warp wait for
// all of them and the chunks of a request would run one warp after another.
GeneratedKernel generate_batch_dispatch(const std::vector<DispatchEntry>& items, int smem_words_per_warp,
                                        int grab = 8);
inline size_t batch_dispatch_smem(int n_programs, int smem_words_per_warp) {
    const size_t head = ((size_t)(n_programs + 1) * 8 + (size_t)n_programs * 12 + 15) & ~(size_t)15;
    return head + (size_t)8 * smem_words_per_warp * 4;
}

// perform_operation: evaluate the program over n rows into the outputs.
GeneratedKernel generate_eval_kernel(const Program& p, const Shape& s);

// One output column of the fused filter kernel: either a gathered frame column
// or an output of the projection program, written compacted.
// ---- aggregate-input expressions fused with the reduction ----------------------------------
// One reduction per slot, over either a program output (an evaluated aggregate input, its
// narrowed value on every row: the reference reduces the evaluated column with null_count 0, so
// its validity is not consulted) or a column of its own (a bare "$k" input; rows whose bit is
// clear are skipped when the column has nulls).
struct AggregateSlot {
    int op = 0;             // GDF_SUM, GDF_MIN or GDF_MAX (AVG reduces as SUM; COUNT needs no kernel)
    bool evaluated = false;
    int index = -1;         // program output, or bare column (index into the bare-column list)
    gdf_dtype dtype = GDF_invalid;  // dtype of the reduced column
    bool skip_nulls = false;
};

// Scratch of an aggregate kernel (zeroed before the launch), 64-bit words: [0] finished-block
// counter, [1 .. S] the results, then grid x S block partials.
inline int64_t aggregate_scratch_words(int slots, int grid) { return 1 + slots + (int64_t)grid * slots; }

// The kernel reads every referenced input once, runs the program per row, folds each slot into a
// per-thread accumulator (integer SUM: int64, wrapping; float SUM: double; MIN / MAX: in the
// column's type with cudf's identities, numeric_limits max / lowest), reduces warps and blocks in
// a fixed order, and the last block folds the block partials in block order: deterministic for a
// given grid.  Param slots: the eval layout, then [counts + 1] = scratch, then the data and the
// validity pointers of the bare columns.
GeneratedKernel generate_aggregate_kernel(const Program& p, const std::vector<AggregateSlot>& slots,
                                          const std::vector<ColumnDesc>& bare, const Shape& s);

struct FilterOutput {
    bool from_project = false;
    int index = -1;          // frame column (gathered) or projection output number
    gdf_dtype dtype = GDF_invalid;
    bool has_valid = false;
};

// The fused LogicalFilter kernel: predicate (a one-output INT8 program, or the
// "$k" clone of a one-byte frame column), single-pass compaction, and the
// compacted write of every output.
struct FilterSpec {
    int n_frame = 0;
    std::vector<gdf_dtype> frame_dtypes;
    std::vector<bool> frame_has_valid;
    bool clone_stencil = false;
    int clone_column = -1;
    const Program* predicate = nullptr;   // inputs are frame columns predicate_cols[i]
    std::vector<int> predicate_cols;
    const Program* project = nullptr;     // optional; inputs are frame columns project_cols[i]
    std::vector<int> project_cols;
    std::vector<FilterOutput> outputs;
};

// Scratch words of a fused filter launch: ticket, error flag, kept-row total,
// one valid-bit count per output, then one look-back status word per tile.
inline int64_t filter_scratch_header(int n_outputs) { return 3 + n_outputs; }

// Rows per look-back tile of a filter kernel with shape s: one warp's chunk of J slices.
inline int64_t filter_tile_rows(const Shape& s) { return (int64_t)32 * s.G * s.J; }

// Widest column the fused filter touches.
int filter_max_width(const FilterSpec& f);

GeneratedKernel generate_filter_kernel(const FilterSpec& f, const Shape& s, bool item = false);

// C type name of a column element.
const char* element_ctype(gdf_dtype t);

// ---- delimited-text scan fused with its filter ---------------------------------------------
// The scanned frame is the projected file columns (BindableTableScan projects=[...]); the
// predicate (optional) reads scanned-frame columns predicate_cols.  Every output carries a mask.
struct TextScanSpec {
    std::vector<gdf_dtype> dtypes;       // per projected column
    std::vector<int> file_cols;          // file column of each projected column
    const Program* predicate = nullptr;  // the LogicalFilter's program, or none (the scan alone)
    std::vector<int> predicate_cols;     // scanned-frame column of each predicate input
};
// Scratch of a text scan launch: ticket, look-back error, kept rows, one valid count per output,
// refused fields, rows past the outputs' capacity; then one status word per chunk.
inline int64_t text_scan_header(int n_outputs) { return 5 + n_outputs; }
// Parameter slots before the outputs: lines, text, bytes, terminator positions, terminators,
// rows skipped, delimiter, output capacity, output row base (0 .. 31: kept row j is written at
// row base + j of the output pointers and masks, which a piece of a longer scan appends into a
// mask word the rows before it have started).
constexpr int kTextScanFixedSlots = 9;
// Lines per look-back chunk of a text scan kernel: J mask words of 32 lines.
inline int64_t text_scan_chunk_lines(const Shape& s) { return (int64_t)32 * s.J; }

GeneratedKernel generate_text_scan_kernel(const TextScanSpec& t, const Shape& s);

}  // namespace ral
