"""ralgpu — Python access to the GB300 expression path through its C ABI.

Mirrors the reference's expression-path API (perform_operation,
evaluate_expression, process_filter, execute_project_plan,
materialize_column, add_expression_to_plan) over gdf_column structures whose
buffers are device memory held by torch tensors.  Every call goes through
libralgpu.so (include/ral/ral_c.h); there is no CPU or torch fallback: if the
library is missing the import of the first entry point raises.
"""
from .capi import (RalError, lib, perform_operation, perform_operation_async, perform_operation_host, evaluate_expression,
                   process_filter, execute_project_plan, filter_project, project_output_types,
                   materialize_column, materialize_columns, apply_boolean_mask, add_expression_to_plan,
                   get_output_type_expression,
                   debug_program_source, debug_filter_source, jit_stats, kernel_launches, version,
                   parse_project_plan, Batch, autotune_program, batch_tune_key, Server, softfp_selftest,
                   debug_lookback_timeout, process_aggregate, debug_aggregate_source, call_timing, filter_grid_launches,
                   Category, category_column, decode_category, filter_project_host,
                   text_scan_rows, text_scan_filter, debug_text_scan_source, parquet_schema,
                   parquet_scan_filter)
from .column import Column, Scalar, valid_alloc_size
from . import dtypes

__all__ = [
    "RalError", "lib", "perform_operation", "perform_operation_async", "perform_operation_host", "evaluate_expression",
    "process_filter", "execute_project_plan", "filter_project", "project_output_types",
    "materialize_column", "materialize_columns", "apply_boolean_mask", "add_expression_to_plan", "get_output_type_expression",
    "debug_program_source", "debug_filter_source", "jit_stats", "kernel_launches", "version", "Column", "Scalar",
    "valid_alloc_size", "dtypes", "parse_project_plan", "Batch", "autotune_program", "batch_tune_key", "Server", "softfp_selftest", "debug_lookback_timeout",
    "process_aggregate", "debug_aggregate_source", "call_timing", "filter_grid_launches", "Category", "category_column",
    "decode_category", "filter_project_host", "text_scan_rows", "text_scan_filter", "debug_text_scan_source",
    "parquet_schema", "parquet_scan_filter",
]
