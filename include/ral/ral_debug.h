/*
 * ral_debug.h — test and introspection hooks of libralgpu.so.
 *
 * NOT part of the drop-in API: a reference-side integration binds only the entry points of
 * ral_c.h.  These functions show the code the library generates, compile it without a GPU,
 * check the integer-pipe double arithmetic on a device and exercise the bounded look-back wait;
 * the library's own tests and tools use them.  Same conventions as ral_c.h (status codes,
 * ral_last_error()).
 */
#ifndef RAL_DEBUG_H_
#define RAL_DEBUG_H_

#include "ral/ral_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Library introspection (no reference counterpart): generated CUDA source of
 * the kernel a program maps to, and an NVRTC-only compile check that needs
 * no GPU.  Buffers receive a NUL-terminated string truncated to capacity. */
int ral_debug_program_source(const gdf_dtype *input_dtypes, const int32_t *input_nullable, int32_t num_inputs,
                             const gdf_dtype *output_dtypes, const int32_t *output_nullable, int32_t num_outputs,
                             const column_index_type *left_inputs, const column_index_type *right_inputs,
                             const column_index_type *outputs, int32_t num_operations,
                             const column_index_type *final_output_positions, const int32_t *operators,
                             const int32_t *unary_operators, const gdf_scalar *left_scalars,
                             const gdf_scalar *right_scalars, int32_t compile, char *source_out,
                             int64_t source_capacity, char *log_out, int64_t log_capacity);

/* Generated source of the batch kernel for the programs added so far (and an NVRTC-only
 * compile when compile != 0); needs no GPU. */
int ral_batch_debug_source(const ral_batch *batch, int32_t compile, char *source_out, int64_t source_capacity,
                           char *log_out, int64_t log_capacity);

/* Generated source of the fused LogicalFilter kernel (optionally NVRTC-compiled, no GPU
 * needed) for a frame described by dtypes and mask presence; project_query_part may be
 * NULL (process_filter) or a LogicalProject (ral_filter_project). */
int ral_debug_filter_source(const gdf_dtype *frame_dtypes, const int32_t *frame_nullable, int32_t num_columns,
                            const char *filter_query_part, const char *project_query_part, int32_t compile,
                            char *source_out, int64_t source_capacity, char *log_out, int64_t log_capacity);

/* Generated source of the fused aggregate kernel of a LogicalAggregate over a frame described by
 * dtypes, mask presence and null counts (optionally NVRTC-compiled, no GPU needed); an empty
 * source when the plan needs no kernel (COUNT only). */
int ral_debug_aggregate_source(const gdf_dtype *frame_dtypes, const int32_t *frame_nullable,
                               const int64_t *frame_null_counts, int32_t num_columns, const char *query_part,
                               int32_t compile, char *source_out, int64_t source_capacity, char *log_out,
                               int64_t log_capacity);

/* Per-call timing of the synchronous filter entry points (ral_process_filter, ral_filter_project):
 * enable != 0 turns it on (also RAL_CALL_TIMING=1), reset != 0 clears it after reading.  *calls
 * receives the calls timed and us4 their mean host preparation (entry to the first enqueue),
 * enqueue, wait for completion and kernel device time, in microseconds. */
int ral_debug_call_timing(int32_t enable, int32_t reset, int64_t *calls, double *us4);

/* Fused filter launches that ran in grid mode (synchronous calls of at most 8Mi rows whose blocks
 * all fit on the device: one cooperative launch, a grid barrier in place of the look-back). */
int ral_debug_filter_grid_launches(int64_t *launches);

/* Generated source of the text scan kernel for a file schema, projections and filter (NULL: none),
 * with an NVRTC-only compile when compile != 0 (log_out gets the ptxas log); needs no GPU. */
int ral_debug_text_scan_source(const int32_t *file_dtypes, int32_t n_file_columns, const int32_t *projections,
                               int32_t n_projections, const char *filter_query_part, int32_t compile, char *source_out,
                               int64_t source_capacity, char *log_out, int64_t log_capacity);

/* Compiles every query's chunk function and links the dispatcher without loading it (no GPU
 * needed); the ptxas / link log goes to log_out. */
int ral_server_debug_compile(ral_server *server, char *log_out, int64_t log_capacity);

/* Served-loop counters beside ral_server_stats: requests run alone on the standalone fused kernel
 * (tables of at least RAL_SERVER_SOLO_ROWS rows), and the seconds summed over completed requests
 * from submission to first launch (queue_s) and from first launch to completion (run_s). */
int ral_server_debug_stats(ral_server *server, int64_t *solo_requests, double *queue_s, double *run_s);

/*
 * Device self-test of the integer-pipe double operations against the GPU's FP64 instructions
 * (no reference counterpart): n random operand sets from seed; mismatches[16] receives the
 * mismatch count of each operation (0 div, 1 floor, 2 ceil, 3 compares, 4 int64->double,
 * 5 double->int64, 6 float->double, 7 double->float, 8 == 0, 9 fabs, 10 int64 / and %,
 * 11 sin / cos beyond 2 ulp of the library's) and first_operands[32]
 * the bits of each operation's first mismatching operands.
 */
int ral_softfp_selftest(int64_t n, uint64_t seed, int64_t *mismatches, uint64_t *first_operands);

/*
 * Failure-detection check (no reference counterpart): runs the compaction over n_rows rows with its
 * tile counter starting at 1, so that tile 1's look-back waits on a status word nothing writes;
 * the bounded wait must end (about a second) with the error word set, reported as
 * *status = RAL_ERROR_TIMEOUT, and the context must stay usable: the same compaction is then run
 * normally and *kept_after receives its kept-row count (n_rows).  n_rows: one tile (4096) < n_rows
 * <= 64M.
 */
int ral_debug_lookback_timeout(int64_t n_rows, int32_t *status, int64_t *kept_after);

#ifdef __cplusplus
}
#endif

#endif /* RAL_DEBUG_H_ */
