/*
 * ral_c.h — C ABI of the GB300 expression-evaluation library (libralgpu.so).
 *
 * These entry points replace the BlazingSQL RAL's expression path.  Each one
 * names the reference interface it stands in for (paths relative to the
 * reference project root).  Conventions:
 *   - Every function returns RAL_SUCCESS (0) or an error code; the message of
 *     the last failure on the calling thread is ral_last_error().  (The
 *     reference throws std::runtime_error; include/ral/ral.hpp rethrows.)
 *   - Columns are gdf_column (include/ral/gdf_compat.h).  Data and validity
 *     buffers are device memory.  Validity buffers must be 4-byte aligned and
 *     hold gdf_valid_allocation_size(size) bytes, as the reference allocates
 *     them: kernels read and write whole 32-bit words.
 *   - Synchronous entry points return after the GPU work is complete, like the
 *     reference.  *_async variants take a cudaStream_t (as void*) and return
 *     after enqueueing.
 *   - Entry points are thread-safe.
 */
#ifndef RAL_C_H_
#define RAL_C_H_

#include "ral/gdf_compat.h"

#ifdef __cplusplus
extern "C" {
#endif

#define RAL_SUCCESS 0
#define RAL_ERROR_INVALID_ARGUMENT 1
#define RAL_ERROR_UNSUPPORTED 2 /* a program or expression the interpreter cannot run */
#define RAL_ERROR_CUDA 3
#define RAL_ERROR_JIT 4
#define RAL_ERROR_ALLOC 5
#define RAL_ERROR_TIMEOUT 6     /* a bounded device-side wait gave up */
#define RAL_ERROR_PARSE 7

const char *ral_last_error(void);
const char *ral_version(void);

/*
 * perform_operation — src/Interpreter/interpreter_cpp.h:25-37
 * (implementation src/Interpreter/interpreter_cpp.cu:219-286).
 * Runs one register program over n = input_columns[0]->size rows into the
 * caller-allocated output columns.  Arrays left_inputs .. right_scalars have
 * num_operations entries; final_output_positions has num_outputs entries.
 * new_input_indices is accepted and ignored, as in the reference.  Output
 * null_count is not updated (the reference leaves it too).
 */
int ral_perform_operation(gdf_column *const *output_columns, int32_t num_outputs,
                          gdf_column *const *input_columns, int32_t num_inputs,
                          const column_index_type *left_inputs, const column_index_type *right_inputs,
                          const column_index_type *outputs, int32_t num_operations,
                          const column_index_type *final_output_positions,
                          const int32_t *operators /* gdf_binary_operator */,
                          const int32_t *unary_operators /* gdf_unary_operator */,
                          const gdf_scalar *left_scalars, const gdf_scalar *right_scalars,
                          const column_index_type *new_input_indices, int32_t num_new_input_indices);

/* Same, enqueued on `stream` (cudaStream_t); when null_counts is non-null the
 * call synchronises and stores each output's null count there (the fused
 * form of execute_project_plan's update_null_count, CalciteInterpreter.cpp:332-335). */
int ral_perform_operation_async(gdf_column *const *output_columns, int32_t num_outputs,
                                gdf_column *const *input_columns, int32_t num_inputs,
                                const column_index_type *left_inputs, const column_index_type *right_inputs,
                                const column_index_type *outputs, int32_t num_operations,
                                const column_index_type *final_output_positions, const int32_t *operators,
                                const int32_t *unary_operators, const gdf_scalar *left_scalars,
                                const gdf_scalar *right_scalars, void *stream, int64_t *null_counts);

/*
 * perform_operation over columns in HOST memory (no reference counterpart; the reference's
 * perform_operation, src/Interpreter/interpreter_cpp.h:25-37, takes device columns).  The
 * gdf_column data and valid pointers are host pointers; the rows stream through the GPU in chunks
 * of chunk_rows (rounded up to a multiple of 1024; 0 = 4Mi rows), each chunk's copies to the
 * device, kernel and copies back on one of three streams, so that copies in both directions
 * overlap the kernels.  Same results as perform_operation over device copies of the columns;
 * output null_count is filled in.  Page-locked host buffers are needed for the overlap.
 * Synchronous.
 */
int ral_perform_operation_host(gdf_column *const *output_columns, int32_t num_outputs,
                               gdf_column *const *input_columns, int32_t num_inputs,
                               const column_index_type *left_inputs, const column_index_type *right_inputs,
                               const column_index_type *outputs, int32_t num_operations,
                               const column_index_type *final_output_positions, const int32_t *operators,
                               const int32_t *unary_operators, const gdf_scalar *left_scalars,
                               const gdf_scalar *right_scalars, int64_t chunk_rows);

/*
 * evaluate_expression — src/LogicalFilter.h:20-23 (src/LogicalFilter.cpp:271-371).
 * Compiles one Calcite RexNode expression over the frame's columns and
 * evaluates it into `output` (caller-allocated, n rows).  For an expression
 * that is a bare column reference "$k" the reference replaces the output with
 * a clone of column k; here column k's data, mask and null count are copied
 * into `output`, whose dtype must then equal column k's.
 */
int ral_evaluate_expression(gdf_column *const *frame_columns, int32_t num_columns, const char *expression,
                            gdf_column *output);

/*
 * process_filter — src/CalciteInterpreter.cpp:509-573.
 * Evaluates the LogicalFilter condition, keeps the rows whose stencil is valid
 * and nonzero and gathers EVERY frame column, in row order, into out_columns.
 * out_columns[i] must have the dtype of frame column i, data capacity for
 * frame_columns[0]->size rows and, exactly when frame column i has one, a
 * validity buffer of that capacity.  On return each out column's size and
 * null_count are set and *num_rows_out holds the kept row count.
 * One fused kernel: predicate, single-pass ballot/look-back compaction and the
 * gather of all columns.
 */
int ral_process_filter(gdf_column *const *frame_columns, int32_t num_columns, const char *query_part,
                       gdf_column *const *out_columns, gdf_size_type *num_rows_out);
int ral_process_filter_async(gdf_column *const *frame_columns, int32_t num_columns, const char *query_part,
                             gdf_column *const *out_columns, gdf_size_type *num_rows_out, void *stream);

/*
 * execute_project_plan — src/CalciteInterpreter.cpp:311-336 with
 * parse_project_plan :123-309.  All evaluated expressions of the
 * LogicalProject run as one program.  out_columns has one entry per projected
 * expression: for a pass-through "$k" the entry is filled with frame column k's
 * buffers (shared, not copied, like the reference); for an evaluated
 * expression the caller provides data (and validity, always expected, as the
 * reference allocates it) of the dtype ral_project_output_types reports.
 * null_count of every output is set.
 */
int ral_project_output_types(const gdf_dtype *frame_dtypes, int32_t num_columns, const char *query_part,
                             int32_t *num_projected, gdf_dtype *dtypes_out, int32_t *is_evaluated_out,
                             int32_t capacity);
int ral_execute_project_plan(gdf_column *const *frame_columns, int32_t num_columns, const char *query_part,
                             gdf_column *const *out_columns, int32_t num_out_columns);

/*
 * parse_project_plan — src/CalciteInterpreter.cpp:123-309 (project_plan_params,
 * src/CalciteInterpreter.h:17-32): the program of a LogicalProject over a frame of the given
 * dtypes.  Receives the frame columns the program reads (dense order), the dtype of each
 * evaluated expression and the op arrays; arrays have room for capacity_ops ops and
 * capacity_cols columns / expressions.
 */
int ral_parse_project_plan(const gdf_dtype *frame_dtypes, int32_t num_columns, const char *query_part,
                           int32_t capacity_ops, int32_t capacity_cols, int32_t *num_input_columns,
                           int32_t *input_columns, int32_t *num_evaluated, gdf_dtype *evaluated_dtypes,
                           int32_t *num_operations, column_index_type *left_inputs, column_index_type *right_inputs,
                           column_index_type *outputs, column_index_type *final_output_positions,
                           int32_t *operators, int32_t *unary_operators, gdf_scalar *left_scalars,
                           gdf_scalar *right_scalars);

/*
 * LogicalFilter followed by LogicalProject, fused (the plan shape
 * "LogicalProject(...)\n  LogicalFilter(condition=[...])", evaluated by
 * CalciteInterpreter.cpp:719-723 as process_filter then execute_project_plan).
 * The projection is evaluated only on kept rows and written compacted; no
 * filtered copy of the frame is materialised.  out_columns as for
 * ral_execute_project_plan but with capacity for frame_columns[0]->size rows;
 * pass-through columns are gathered (not shared).
 */
int ral_filter_project(gdf_column *const *frame_columns, int32_t num_columns, const char *filter_query_part,
                       const char *project_query_part, gdf_column *const *out_columns, int32_t num_out_columns,
                       gdf_size_type *num_rows_out);

/*
 * process_filter / the fused LogicalFilter + LogicalProject over columns in HOST memory (no
 * reference counterpart: the reference's process_filter, src/CalciteInterpreter.cpp:509-573, works
 * on device columns).  frame_columns and out_columns hold host pointers (page-locked for overlap);
 * project_query_part NULL filters the frame (every column gathered, out_columns as for
 * ral_process_filter), otherwise out_columns are as for ral_filter_project.  The rows stream
 * through the GPU in chunks of chunk_rows (rounded up to a multiple of 1024; 0 = 4Mi rows) on three
 * streams: each chunk's copies in, the fused filter kernel, and its kept rows copied back to their
 * place in the outputs, overlapping the other chunks' copies.  Same results as the device entry
 * points; sizes and null counts are set.  A string literal missing from a category column's
 * dictionary is refused (adding it would rewrite the column, which lives in host memory).
 * Synchronous.
 */
int ral_filter_project_host(gdf_column *const *frame_columns, int32_t num_columns, const char *filter_query_part,
                            const char *project_query_part, gdf_column *const *out_columns, int32_t num_out_columns,
                            gdf_size_type *num_rows_out, int64_t chunk_rows);

/*
 * materialize_column — src/ColumnManipulation.cuh:16-18 (ColumnManipulation.cu:137-150).
 * output[i] = input[row_indices[i]] for row_indices[i] >= 0; valid bit i =
 * valid bit row_indices[i] (0 for a negative index); output->null_count is
 * recounted.  row_indices is an INT8/16/32/64 column.
 */
int ral_materialize_column(const gdf_column *input, gdf_column *output, const gdf_column *row_indices);

/*
 * materialize_column over many columns at once — the callers that gather every column of a table
 * by the same index column: joins (src/operators/JoinOperator.cpp:130,135), order-by
 * (src/operators/OrderBy.cpp:66) and the distribution primitives (src/distribution/primitives.cpp:
 * 239,426,667) call materialize_column once per column.  Same per-column result as
 * ral_materialize_column (including the recounted null_count and size of every output); the
 * index column is read once for all columns, in one kernel.  All inputs must have the same size;
 * 0 <= num_columns <= 64.
 */
int ral_materialize_columns(const gdf_column *const *inputs, gdf_column *const *outputs, int32_t num_columns,
                            const gdf_column *row_indices);

/*
 * apply_boolean_mask over the row-index column — src/CalciteInterpreter.cpp:531-543
 * (gdf_sequence iota + cudf::apply_boolean_mask).  Writes, in row order, the
 * indices of the rows whose stencil byte is nonzero and whose stencil validity
 * bit is set (stencil->valid may be NULL) into out_indices (INT32, capacity
 * stencil->size rows) and sets out_indices->size and *num_rows_out.  stencil is
 * an INT8 or BOOL8 column.  Single-pass compaction (ballot/popc, block scan,
 * decoupled look-back); the look-back state lives in scratch memory this call
 * allocates and frees on the stream.
 */
int ral_apply_boolean_mask(const gdf_column *stencil, gdf_column *out_indices, gdf_size_type *num_rows_out);

/*
 * ral_apply_boolean_mask_noalloc — no counterpart in the reference.
 * The same result as ral_apply_boolean_mask, for callers that cannot allocate
 * device memory (an engine whose pool already owns the whole GPU, or a
 * latency-critical path that must not enter the driver's allocator): the
 * scratch block comes from a fixed 256 KiB array compiled into the library,
 * which every GPU that loads the library holds until the process exits.
 * Limit: stencil->size <= RAL_NOALLOC_MAX_ROWS; larger stencils are rejected
 * with RAL_ERROR_INVALID_ARGUMENT.  Each call looks up the array's device
 * address on the current device (cudaGetSymbolAddress); the first call on a
 * device also loads the library's module there, so make that first call before
 * any stream capture.  All calls share the array: calls whose GPU work
 * overlaps (from several threads or streams at once) race on it.
 */
#define RAL_NOALLOC_MAX_ROWS ((int64_t)(256 * 1024 / 8 - 3) * 4096)
int ral_apply_boolean_mask_noalloc(const gdf_column *stencil, gdf_column *out_indices, gdf_size_type *num_rows_out);

/*
 * process_aggregate without GROUP BY — src/operators/GroupBy.cpp:531-590 with compute_aggregations
 * (:298-345) and aggregations_without_groupby (:231-296).  query_part is the LogicalAggregate
 * ("LogicalAggregate(group=[{}], EXPR$0=[SUM(*($0, $1))], EXPR$1=[COUNT()], ...)"); each
 * aggregation is SUM, MIN, MAX, AVG or COUNT of an expression over the frame or of a bare "$k".
 * The reference evaluates every expression input into a full column and then reduces it; here all
 * expression inputs run as one register program whose results are reduced in the same kernel, so
 * no intermediate column is written.  results[i] receives aggregation i as the reference's one-row
 * output column holds it (dtype by get_aggregation_output_type, CalciteExpressionParsing.cpp:92-116;
 * is_valid false where the reference returns a null); *num_results the aggregation count.
 * Results match the reference's flow: an evaluated input's nulls are not skipped (evaluate_expression
 * leaves its null_count at 0), a bare input's are; COUNT() counts column 0's non-null rows.
 * Float sums are deterministic on a given GPU but their rounding follows a tree order, not a
 * sequential one.  A GROUP BY plan returns RAL_ERROR_UNSUPPORTED.  Synchronous.
 */
int ral_process_aggregate(gdf_column *const *frame_columns, int32_t num_columns, const char *query_part,
                          gdf_scalar *results, int32_t capacity, int32_t *num_results);

/*
 * Scan -> filter fusion over delimited text — a BindableTableScan of a CSV table
 * (src/CalciteInterpreter.cpp:745-767: `projects=[...]` picks the file columns, loaded through
 * csv_parser::parse, src/io/data_parser/CSVParser.cpp:176-233, with '|' as the default delimiter,
 * no header, blank lines skipped) followed by its LogicalFilter (src/CalciteInterpreter.cpp:509),
 * evaluated while the text is parsed: only the fields the condition reads are parsed for every
 * row, and the projected fields only for the rows kept.
 *
 * `data` holds n_bytes of text in device memory.  Lines end at line_terminator (the last may lack
 * it; a '\r' before it is dropped); the first skip_rows lines are skipped and blank lines are not
 * rows.  file_dtypes gives the file's n_file_columns column types (INT8/16/32/64, FLOAT32/64,
 * DATE32, DATE64); projections lists the file column of each scanned column, in the scan's order.
 * filter_query_part is the LogicalFilter text over the scanned columns ($k = k-th projection), or
 * NULL for the scan alone.  out_columns: one per projection, of the file column's dtype, with a
 * validity mask (4-byte aligned) and size = capacity in rows (ral_text_scan_rows gives the number
 * of rows); on return size = rows kept and null_count set.  Field rules (empty or unreadable
 * fields are null; decimals rounded to nearest, refused with RAL_ERROR_UNSUPPORTED where the
 * exact method does not reach; dates YYYY-MM-DD[ HH:MM:SS]) are those of csrc/textscan.cuh.
 * Synchronous.
 */
int ral_text_scan_rows(const char *data, int64_t n_bytes, char line_terminator, int32_t skip_rows, int64_t *rows);
int ral_text_scan_filter(const char *data, int64_t n_bytes, char delimiter, char line_terminator, int32_t skip_rows,
                         const int32_t *file_dtypes, int32_t n_file_columns, const int32_t *projections,
                         int32_t n_projections, const char *filter_query_part, gdf_column *const *out_columns,
                         gdf_size_type *num_rows_out);
/* The same with `text` in host memory (page-locked for full speed): the text goes to the device in
 * pieces of whole lines (64 MiB by default), each scanned while the next ones are copied, the kept
 * rows appended to out_columns in order.  Same arguments, results and errors. */
int ral_text_scan_filter_host(const char *text, int64_t n_bytes, char delimiter, char line_terminator,
                              int32_t skip_rows, const int32_t *file_dtypes, int32_t n_file_columns,
                              const int32_t *projections, int32_t n_projections, const char *filter_query_part,
                              gdf_column *const *out_columns, gdf_size_type *num_rows_out);

/*
 * The same fusion over a Parquet file — a BindableTableScan of a Parquet table (parquet_parser::parse,
 * src/io/data_parser/ParquetParser.cpp:36-90, cudf's Parquet reader) followed by its LogicalFilter.
 * `file` holds the whole file (n_bytes) in host memory.  In page-locked memory the decode kernels read
 * the projected pages in place over the host link; otherwise the projected leaves' column chunks
 * are copied in, in batches decoded while the next batch is copied.  Snappy pages are decompressed
 * on the device (one warp per page), a levels kernel decodes the definition levels of optional
 * leaves, a dictionary kernel the indices of dictionary-encoded pages, a values kernel every page's
 * values in 8192-row items, and the fused filter kernel filters the decoded columns.
 * ral_parquet_schema gives the row count, the leaf count and the gdf dtype each leaf scans as
 * (GDF_invalid where unsupported; dtypes: host array of `capacity` entries).
 * Supported: flat schemas; INT32 (DATE as DATE32), INT64 (TIMESTAMP_MILLIS as DATE64), FLOAT,
 * DOUBLE; required and optional leaves; v1 and v2 data pages of PLAIN values or dictionary indices
 * (PLAIN_DICTIONARY / RLE_DICTIONARY, with the chunk's PLAIN dictionary page), RLE / bit-packed
 * definition levels; uncompressed or SNAPPY column chunks — anything else returns
 * RAL_ERROR_UNSUPPORTED, as does a page that does not decode within its bytes.  out_columns: one per
 * projection, of its dtype, with a 4-byte aligned mask and room for every row of the file; on return
 * size = rows kept.  Synchronous.
 */
int ral_parquet_schema(const uint8_t *file, int64_t n_bytes, int64_t *rows, int32_t *n_columns, int32_t *dtypes,
                       int32_t capacity);
int ral_parquet_scan_filter(const uint8_t *file, int64_t n_bytes, const int32_t *projections, int32_t n_projections,
                            const char *filter_query_part, gdf_column *const *out_columns, gdf_size_type *num_rows_out);

/*
 * String-category dictionaries — the NVCategory a GDF_STRING_CATEGORY column points at through
 * dtype_info.category in the reference, where a string literal compared with such a column is looked
 * up (src/LogicalFilter.cpp:150-194).  A ral_category keeps its distinct strings sorted by byte
 * value; a column's int32 codes are the ranks of its strings, so comparing codes compares strings.
 * ral_category_create builds one from n strings (duplicates allowed) and writes each string's code
 * to codes_out (host array of n entries; may be NULL).  A filter or projection whose text compares
 * such a column with a string literal ("=($k, 'abc')", literal on the right as the reference
 * requires) uses the literal's code; when the dictionary lacks the string, the call makes a new
 * dictionary with it, rewrites the column's codes to the new ranks on the device and points the
 * column's dtype_info.category at the new dictionary, as the reference does.  The caller owns every
 * dictionary, including ones the library made, and frees them with ral_category_destroy.
 */
typedef struct ral_category_s ral_category;
int ral_category_create(const char *const *strings, int64_t n, ral_category **category, int32_t *codes_out);
int ral_category_size(const ral_category *category, int64_t *num_keys);
/* *code = the string's code, or -1 when the dictionary lacks it (NVCategory::get_value). */
int ral_category_get_value(const ral_category *category, const char *str, int32_t *code);
/* The string of a code, NUL-terminated and truncated to capacity; *length its full byte length. */
int ral_category_key(const ral_category *category, int32_t code, char *buf, int64_t capacity, int64_t *length);
int ral_category_destroy(ral_category *category);

/*
 * add_expression_to_plan — src/LogicalFilter.h:26-42 (src/LogicalFilter.cpp:44-268).
 * The register-program emitter: appends the ops of `expression` to the arrays.
 * *num_operations is in/out (ops already present / after); arrays have room
 * for `capacity` ops.  new_input_indices maps frame column -> dense input
 * register (size num_frame_columns).
 */
int ral_add_expression_to_plan(const char *expression, column_index_type expression_position,
                               column_index_type num_outputs, column_index_type num_inputs,
                               const column_index_type *new_input_indices, int32_t num_frame_columns,
                               column_index_type *left_inputs, column_index_type *right_inputs,
                               column_index_type *outputs, int32_t *operators, int32_t *unary_operators,
                               gdf_scalar *left_scalars, gdf_scalar *right_scalars, int32_t *num_operations,
                               int32_t capacity);

/* get_output_type_expression — src/CalciteExpressionParsing.cpp:420-481. */
int ral_get_output_type_expression(const gdf_dtype *frame_dtypes, int32_t num_columns, const char *expression,
                                   gdf_dtype *dtype_out);

/*
 * Batched execution — no single reference counterpart: the reference runs each program as its
 * own perform_operation call.  A batch holds many perform_operation calls (each over its own
 * columns) and runs them all in ONE persistent kernel whose warps pull (program, row-tile)
 * work items from a device counter; the launch is captured once in a CUDA graph and replayed.
 * Column descriptors are copied at add time; their buffers must stay allocated and in place.
 * Results are identical to calling ral_perform_operation on each program.
 */
typedef struct ral_batch_s ral_batch;
int ral_batch_create(ral_batch **batch);
/* Adds one program with perform_operation's arguments; *program_index receives its index. */
int ral_batch_add(ral_batch *batch, gdf_column *const *output_columns, int32_t num_outputs,
                  gdf_column *const *input_columns, int32_t num_inputs, const column_index_type *left_inputs,
                  const column_index_type *right_inputs, const column_index_type *outputs, int32_t num_operations,
                  const column_index_type *final_output_positions, const int32_t *operators,
                  const int32_t *unary_operators, const gdf_scalar *left_scalars, const gdf_scalar *right_scalars,
                  int32_t *program_index);
/* Picks launch shapes (autotuner table), compiles the batch kernel, uploads work
 * descriptors and captures the CUDA graph.  Optional: ral_batch_run prepares on first use. */
int ral_batch_prepare(ral_batch *batch);
/* Runs every program once on `stream` (NULL: per-thread default stream); use_graph = 0
 * launches the kernel directly instead of replaying the graph.  Asynchronous. */
int ral_batch_run(ral_batch *batch, void *stream, int32_t use_graph);
int ral_batch_info(const ral_batch *batch, int32_t *num_programs, int64_t *total_rows, int64_t *work_items);
int ral_batch_destroy(ral_batch *batch);
/* Registers per thread, grid and resident blocks per SM of the prepared batch kernel (0 before
 * ral_batch_prepare). */
int ral_batch_kernel_info(const ral_batch *batch, int32_t *registers, int32_t *grid, int32_t *blocks_per_sm);

/* The autotuner's table key of a perform_operation program (dtype mix and program length). */
int ral_batch_tune_key(gdf_column *const *output_columns, int32_t num_outputs, gdf_column *const *input_columns,
                       int32_t num_inputs, const column_index_type *left_inputs, const column_index_type *right_inputs,
                       const column_index_type *outputs, int32_t num_operations,
                       const column_index_type *final_output_positions, const int32_t *operators,
                       const int32_t *unary_operators, const gdf_scalar *left_scalars, const gdf_scalar *right_scalars,
                       char *key_out, int64_t key_capacity);

/*
 * Autotuner: runs the perform_operation program as a one-program batch at each candidate tile
 * shape (rows per warp tile 32*G*J for J in 2, 4, 8, 16; slice loop unrolled 1 or 2 times; double
 * operations on the integer pipes or as FP64 instructions), times it and records the fastest in
 * the tuning table (keyed by dtype mix and program length; persisted as JSON in the JIT cache
 * directory), which batches consult.  Writes the program's outputs as a side effect.
 * *best_slices / *best_unroll / *best_soft_fp receive the chosen shape and *best_ms its kernel time.
 */
int ral_autotune_program(gdf_column *const *output_columns, int32_t num_outputs, gdf_column *const *input_columns,
                         int32_t num_inputs, const column_index_type *left_inputs,
                         const column_index_type *right_inputs, const column_index_type *outputs,
                         int32_t num_operations, const column_index_type *final_output_positions,
                         const int32_t *operators, const int32_t *unary_operators, const gdf_scalar *left_scalars,
                         const gdf_scalar *right_scalars, int32_t *best_slices, int32_t *best_unroll,
                         int32_t *best_soft_fp, double *best_ms);

/* Kernels launched by this library since load (all entry points). */
int64_t ral_kernel_launches(void);

/* JIT counters: kernels compiled, disk-cache hits, memory-cache hits, total compile ms. */
int ral_jit_stats(int64_t *compiles, int64_t *disk_hits, int64_t *memory_hits, double *compile_ms);

/*
 * Served execution (no reference counterpart: the reference runs one query at a time).  A
 * server keeps registered tables resident (the caller's device columns, not copied), plans
 * filter + project queries over them, and runs submitted requests with continuous batching:
 * a scheduler thread admits requests while resident tables plus the outputs of admitted
 * requests stay under budget_bytes, and runs them in waves of the persistent dispatcher (up to
 * wave_rows rows each, fewest rows left first, large requests sliced over several waves); up to
 * max_waves waves are in flight at once.
 */
typedef struct ral_server_s ral_server;
/* wave_rows: rows one wave may carry (a large request is sliced over several waves); 0 = 32M. */
int ral_server_create(int64_t budget_bytes, int32_t max_waves, int32_t max_wave_requests, int64_t wave_rows,
                      ral_server **server);
int ral_server_add_table(ral_server *server, gdf_column *const *columns, int32_t num_columns, int32_t *table_id);
/* filter_query_part: "LogicalFilter(condition=[...])"; project_query_part: "LogicalProject(...)". */
int ral_server_add_query(ral_server *server, int32_t table_id, const char *filter_query_part,
                         const char *project_query_part, int32_t *query_id);
/* dtype and mask presence (0/1) of each projected column; *num_outputs receives the count. */
int ral_server_query_outputs(ral_server *server, int32_t query_id, gdf_dtype *dtypes, int32_t *has_valid,
                             int32_t capacity, int32_t *num_outputs);
/* Compiles every query, links the dispatcher and starts the scheduler thread. */
int ral_server_start(ral_server *server);
/* keep != 0: the outputs stay allocated for ral_server_result until ral_server_release. */
int ral_server_submit(ral_server *server, int32_t query_id, int32_t keep, int64_t *request_id);
/* Blocks up to timeout_s; *latency_s is submit-to-completion on the server's clock. */
int ral_server_wait(ral_server *server, int64_t request_id, double timeout_s, int64_t *rows_out, double *latency_s);
/* Descriptors of a kept request's outputs (device memory owned by the server). */
int ral_server_result(ral_server *server, int64_t request_id, gdf_column *out_columns, int32_t num_outputs);
/* Copies a kept request's outputs into the caller's columns (device buffers of at least the
 * kept row count; masks 64-byte padded) and sets their size and null_count. */
int ral_server_copy_result(ral_server *server, int64_t request_id, gdf_column *const *out_columns,
                           int32_t num_outputs);
int ral_server_release(ral_server *server, int64_t request_id);
/* Submits request k (query queries[k]) at arrival_s[k] seconds after the call starts, waits for
 * all, and fills each latency (from the scheduled arrival to completion) and kept row count. */
int ral_server_run_trace(ral_server *server, int32_t num_requests, const int32_t *queries, const double *arrival_s,
                         double *latency_s, int64_t *rows_out, double *makespan_s);
/* stats: submitted, completed, waves, largest wave, peak reserved bytes, busy microseconds. */
int ral_server_stats(ral_server *server, int64_t *stats6);
int ral_server_destroy(ral_server *server);

#ifdef __cplusplus
}
#endif

#endif /* RAL_C_H_ */
