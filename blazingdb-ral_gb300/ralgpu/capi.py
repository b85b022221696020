"""ctypes bindings of include/ral/ral_c.h and Python-shaped entry points."""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import dtypes as D
from .column import Column, GdfColumn, GdfScalar, Scalar

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "libralgpu.so")
_lib = None

C = ctypes
P = C.c_void_p
I16P = C.POINTER(C.c_int16)
I32P = C.POINTER(C.c_int32)
COLPP = C.POINTER(C.POINTER(GdfColumn))
SCP = C.POINTER(GdfScalar)

_SIGS = {
    "ral_last_error": (C.c_char_p, []),
    "ral_version": (C.c_char_p, []),
    "ral_perform_operation": (C.c_int, [COLPP, C.c_int32, COLPP, C.c_int32, I16P, I16P, I16P, C.c_int32, I16P,
                                        I32P, I32P, SCP, SCP, I16P, C.c_int32]),
    "ral_perform_operation_host": (C.c_int, [COLPP, C.c_int32, COLPP, C.c_int32, I16P, I16P, I16P, C.c_int32, I16P,
                                             I32P, I32P, SCP, SCP, C.c_int64]),
    "ral_perform_operation_async": (C.c_int, [COLPP, C.c_int32, COLPP, C.c_int32, I16P, I16P, I16P, C.c_int32,
                                              I16P, I32P, I32P, SCP, SCP, P, C.POINTER(C.c_int64)]),
    "ral_evaluate_expression": (C.c_int, [COLPP, C.c_int32, C.c_char_p, C.POINTER(GdfColumn)]),
    "ral_process_filter": (C.c_int, [COLPP, C.c_int32, C.c_char_p, COLPP, C.POINTER(C.c_int32)]),
    "ral_process_filter_async": (C.c_int, [COLPP, C.c_int32, C.c_char_p, COLPP, C.POINTER(C.c_int32), P]),
    "ral_project_output_types": (C.c_int, [I32P, C.c_int32, C.c_char_p, I32P, I32P, I32P, C.c_int32]),
    "ral_execute_project_plan": (C.c_int, [COLPP, C.c_int32, C.c_char_p, COLPP, C.c_int32]),
    "ral_filter_project": (C.c_int, [COLPP, C.c_int32, C.c_char_p, C.c_char_p, COLPP, C.c_int32,
                                     C.POINTER(C.c_int32)]),
    "ral_apply_boolean_mask": (C.c_int, [C.POINTER(GdfColumn), C.POINTER(GdfColumn), C.POINTER(C.c_int32)]),
    "ral_materialize_column": (C.c_int, [C.POINTER(GdfColumn), C.POINTER(GdfColumn), C.POINTER(GdfColumn)]),
    "ral_materialize_columns": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(GdfColumn)]),
    "ral_add_expression_to_plan": (C.c_int, [C.c_char_p, C.c_int16, C.c_int16, C.c_int16, I16P, C.c_int32,
                                             I16P, I16P, I16P, I32P, I32P, SCP, SCP, I32P, C.c_int32]),
    "ral_get_output_type_expression": (C.c_int, [I32P, C.c_int32, C.c_char_p, I32P]),
    "ral_debug_program_source": (C.c_int, [I32P, I32P, C.c_int32, I32P, I32P, C.c_int32, I16P, I16P, I16P,
                                           C.c_int32, I16P, I32P, I32P, SCP, SCP, C.c_int32, C.c_char_p,
                                           C.c_int64, C.c_char_p, C.c_int64]),
    "ral_kernel_launches": (C.c_int64, []),
    "ral_debug_filter_source": (C.c_int, [I32P, I32P, C.c_int32, C.c_char_p, C.c_char_p, C.c_int32, C.c_char_p,
                                          C.c_int64, C.c_char_p, C.c_int64]),
    "ral_debug_aggregate_source": (C.c_int, [I32P, I32P, C.c_void_p, C.c_int32, C.c_char_p, C.c_int32, C.c_char_p,
                                             C.c_int64, C.c_char_p, C.c_int64]),
    "ral_process_aggregate": (C.c_int, [C.c_void_p, C.c_int32, C.c_char_p, C.POINTER(GdfScalar), C.c_int32,
                                        C.POINTER(C.c_int32)]),
    "ral_debug_call_timing": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "ral_debug_filter_grid_launches": (C.c_int, [C.POINTER(C.c_int64)]),
    "ral_text_scan_rows": (C.c_int, [C.c_void_p, C.c_int64, C.c_char, C.c_int32, C.POINTER(C.c_int64)]),
    "ral_text_scan_filter": (C.c_int, [C.c_void_p, C.c_int64, C.c_char, C.c_char, C.c_int32, I32P, C.c_int32, I32P,
                                       C.c_int32, C.c_char_p, C.c_void_p, C.POINTER(C.c_int32)]),
    "ral_text_scan_filter_host": (C.c_int, [C.c_void_p, C.c_int64, C.c_char, C.c_char, C.c_int32, I32P, C.c_int32,
                                            I32P, C.c_int32, C.c_char_p, C.c_void_p, C.POINTER(C.c_int32)]),
    "ral_debug_text_scan_source": (C.c_int, [I32P, C.c_int32, I32P, C.c_int32, C.c_char_p, C.c_int32, C.c_char_p,
                                             C.c_int64, C.c_char_p, C.c_int64]),
    "ral_parquet_schema": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int32), I32P,
                                     C.c_int32]),
    "ral_parquet_scan_filter": (C.c_int, [C.c_void_p, C.c_int64, I32P, C.c_int32, C.c_char_p, C.c_void_p,
                                          C.POINTER(C.c_int32)]),
    "ral_filter_project_host": (C.c_int, [C.c_void_p, C.c_int32, C.c_char_p, C.c_char_p, C.c_void_p, C.c_int32,
                                          C.POINTER(C.c_int32), C.c_int64]),
    "ral_category_create": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_void_p), I32P]),
    "ral_category_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "ral_category_get_value": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int32)]),
    "ral_category_key": (C.c_int, [C.c_void_p, C.c_int32, C.c_char_p, C.c_int64, C.POINTER(C.c_int64)]),
    "ral_category_destroy": (C.c_int, [C.c_void_p]),
    "ral_jit_stats": (C.c_int, [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                C.POINTER(C.c_double)]),
    "ral_parse_project_plan": (C.c_int, [I32P, C.c_int32, C.c_char_p, C.c_int32, C.c_int32, I32P, I32P, I32P, I32P,
                                         I32P, I16P, I16P, I16P, I16P, I32P, I32P, SCP, SCP]),
    "ral_batch_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "ral_batch_add": (C.c_int, [P, COLPP, C.c_int32, COLPP, C.c_int32, I16P, I16P, I16P, C.c_int32, I16P, I32P, I32P,
                                SCP, SCP, I32P]),
    "ral_batch_prepare": (C.c_int, [P]),
    "ral_batch_run": (C.c_int, [P, P, C.c_int32]),
    "ral_batch_info": (C.c_int, [P, I32P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "ral_batch_debug_source": (C.c_int, [P, C.c_int32, C.c_char_p, C.c_int64, C.c_char_p, C.c_int64]),
    "ral_batch_destroy": (C.c_int, [P]),
    "ral_batch_kernel_info": (C.c_int, [P, I32P, I32P, I32P]),
    "ral_server_create": (C.c_int, [C.c_int64, C.c_int32, C.c_int32, C.c_int64, C.POINTER(C.c_void_p)]),
    "ral_server_add_table": (C.c_int, [P, COLPP, C.c_int32, I32P]),
    "ral_server_add_query": (C.c_int, [P, C.c_int32, C.c_char_p, C.c_char_p, I32P]),
    "ral_server_query_outputs": (C.c_int, [P, C.c_int32, I32P, I32P, C.c_int32, I32P]),
    "ral_server_start": (C.c_int, [P]),
    "ral_server_debug_compile": (C.c_int, [P, C.c_char_p, C.c_int64]),
    "ral_server_submit": (C.c_int, [P, C.c_int32, C.c_int32, C.POINTER(C.c_int64)]),
    "ral_server_wait": (C.c_int, [P, C.c_int64, C.c_double, C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "ral_server_result": (C.c_int, [P, C.c_int64, C.POINTER(GdfColumn), C.c_int32]),
    "ral_server_release": (C.c_int, [P, C.c_int64]),
    "ral_server_copy_result": (C.c_int, [P, C.c_int64, COLPP, C.c_int32]),
    "ral_server_run_trace": (C.c_int, [P, C.c_int32, I32P, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "ral_server_stats": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "ral_server_debug_stats": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ral_server_destroy": (C.c_int, [P]),
    "ral_softfp_selftest": (C.c_int, [C.c_int64, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(C.c_uint64)]),
    "ral_debug_lookback_timeout": (C.c_int, [C.c_int64, I32P, C.POINTER(C.c_int64)]),
    "ral_batch_tune_key": (C.c_int, [COLPP, C.c_int32, COLPP, C.c_int32, I16P, I16P, I16P, C.c_int32, I16P, I32P, I32P,
                                     SCP, SCP, C.c_char_p, C.c_int64]),
    "ral_autotune_program": (C.c_int, [COLPP, C.c_int32, COLPP, C.c_int32, I16P, I16P, I16P, C.c_int32, I16P, I32P,
                                       I32P, SCP, SCP, I32P, I32P, I32P, C.POINTER(C.c_double)]),
}


class RalError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def lib():
    """Loads libralgpu.so (built by blazingdb-ral_gb300/build.py); raises if it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise RalError(-1, f"libralgpu.so not built ({_LIB_PATH}); run __graft_entry__.build()")
        L = C.CDLL(_LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RalError(rc, lib().ral_last_error().decode(errors="replace"))


def version() -> str:
    return lib().ral_version().decode()


def _i16(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int16))


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _p16(a: np.ndarray):
    return a.ctypes.data_as(I16P)


def _p32(a: np.ndarray):
    return a.ctypes.data_as(I32P)


def _colarray(cols: Sequence[Column]):
    structs = [c.to_c() for c in cols]
    arr = (C.POINTER(GdfColumn) * max(1, len(structs)))()
    for i, s in enumerate(structs):
        arr[i] = C.pointer(s)
    return arr, structs


def _sync_categories(frame: Sequence[Column], structs) -> None:
    """A call that resolved a string literal missing from a category column's dictionary points
    the column at a new dictionary (and rewrote its codes): carry the new address over."""
    for c, st in zip(frame, structs):
        if c.dtype == D.GDF_STRING_CATEGORY and st.dtype_info.category:
            c.category = int(st.dtype_info.category)


def _scalars(ss: Sequence[Scalar]):
    arr = (GdfScalar * max(1, len(ss)))()
    for i, s in enumerate(ss):
        arr[i] = s.to_c()
    return arr


def _as_scalar(s) -> Scalar:
    if isinstance(s, Scalar):
        return s
    if isinstance(s, tuple):
        return Scalar(*s)
    raise TypeError("scalars are ralgpu.Scalar or (dtype, value[, is_valid]) tuples")


def perform_operation(output_columns: List[Column], input_columns: List[Column], left_inputs, right_inputs,
                      outputs, final_output_positions, operators, unary_operators, left_scalars, right_scalars,
                      new_input_indices=None) -> None:
    """perform_operation (src/Interpreter/interpreter_cpp.h:25-37), synchronous."""
    oa, _os = _colarray(output_columns)
    ia, _is = _colarray(input_columns)
    l, r, o, f = _i16(left_inputs), _i16(right_inputs), _i16(outputs), _i16(final_output_positions)
    b, u = _i32(operators), _i32(unary_operators)
    ls = _scalars([_as_scalar(s) for s in left_scalars])
    rs = _scalars([_as_scalar(s) for s in right_scalars])
    nii = _i16(new_input_indices if new_input_indices is not None else list(range(len(input_columns))))
    _check(lib().ral_perform_operation(oa, len(output_columns), ia, len(input_columns), _p16(l), _p16(r), _p16(o),
                                       len(l), _p16(f), _p32(b), _p32(u), ls, rs, _p16(nii), len(nii)))


def perform_operation_host(output_columns: List[Column], input_columns: List[Column], left_inputs, right_inputs,
                           outputs, final_output_positions, operators, unary_operators, left_scalars, right_scalars,
                           chunk_rows: int = 0) -> None:
    """perform_operation over columns whose buffers are in host memory (pinned for overlap); the
    rows stream through the GPU in chunks.  Output null counts are filled in."""
    oa, ostructs = _colarray(output_columns)
    ia, _is = _colarray(input_columns)
    l, r, o, f = _i16(left_inputs), _i16(right_inputs), _i16(outputs), _i16(final_output_positions)
    b, u = _i32(operators), _i32(unary_operators)
    ls = _scalars([_as_scalar(s) for s in left_scalars])
    rs = _scalars([_as_scalar(s) for s in right_scalars])
    _check(lib().ral_perform_operation_host(oa, len(output_columns), ia, len(input_columns), _p16(l), _p16(r),
                                            _p16(o), len(l), _p16(f), _p32(b), _p32(u), ls, rs, int(chunk_rows)))
    for c, st in zip(output_columns, ostructs):
        c.null_count = st.null_count


def perform_operation_async(output_columns: List[Column], input_columns: List[Column], left_inputs, right_inputs,
                            outputs, final_output_positions, operators, unary_operators, left_scalars,
                            right_scalars, stream=None, want_null_counts: bool = False):
    """Enqueues on `stream` (torch.cuda.Stream, raw handle, or None = torch's current stream)."""
    import torch
    if stream is None:
        handle = torch.cuda.current_stream().cuda_stream
    elif isinstance(stream, int):
        handle = stream
    else:
        handle = stream.cuda_stream
    oa, _os = _colarray(output_columns)
    ia, _is = _colarray(input_columns)
    l, r, o, f = _i16(left_inputs), _i16(right_inputs), _i16(outputs), _i16(final_output_positions)
    b, u = _i32(operators), _i32(unary_operators)
    ls = _scalars([_as_scalar(s) for s in left_scalars])
    rs = _scalars([_as_scalar(s) for s in right_scalars])
    nc = np.zeros(len(output_columns), dtype=np.int64)
    ncp = nc.ctypes.data_as(C.POINTER(C.c_int64)) if want_null_counts else None
    _check(lib().ral_perform_operation_async(oa, len(output_columns), ia, len(input_columns), _p16(l), _p16(r),
                                             _p16(o), len(l), _p16(f), _p32(b), _p32(u), ls, rs, C.c_void_p(handle),
                                             ncp))
    if want_null_counts:
        for col, v in zip(output_columns, nc):
            col.null_count = int(v)
        return nc
    return None


def evaluate_expression(frame: List[Column], expression: str, output: Column) -> Column:
    """evaluate_expression (src/LogicalFilter.h:20-23)."""
    fa, _fs = _colarray(frame)
    oc = output.to_c()
    _check(lib().ral_evaluate_expression(fa, len(frame), expression.encode(), C.byref(oc)))
    _sync_categories(frame, _fs)
    output.sync_from_c(oc)
    return output


def process_filter(frame: List[Column], query_part: str) -> List[Column]:
    """LogicalFilter (src/CalciteInterpreter.cpp:509-573): returns the filtered frame (new columns)."""
    n = frame[0].size
    outs = [Column.empty(c.dtype, n, with_valid=c.valid is not None) for c in frame]
    fa, _fs = _colarray(frame)
    oa, ostructs = _colarray(outs)
    n_out = C.c_int32(0)
    _check(lib().ral_process_filter(fa, len(frame), query_part.encode(), oa, C.byref(n_out)))
    _sync_categories(frame, _fs)
    for col, s in zip(outs, ostructs):
        col.sync_from_c(s)
    return outs


def project_output_types(frame_dtypes: Sequence[int], query_part: str) -> Tuple[List[int], List[bool]]:
    fd = _i32(frame_dtypes)
    cap = 4096
    n = C.c_int32(0)
    dt = np.zeros(cap, dtype=np.int32)
    ev = np.zeros(cap, dtype=np.int32)
    _check(lib().ral_project_output_types(_p32(fd), len(fd), query_part.encode(), C.byref(n), _p32(dt), _p32(ev), cap))
    return [int(x) for x in dt[:n.value]], [bool(x) for x in ev[:n.value]]


def execute_project_plan(frame: List[Column], query_part: str) -> List[Column]:
    """LogicalProject (src/CalciteInterpreter.cpp:311-336): returns the projected frame."""
    types, evald = project_output_types([c.dtype for c in frame], query_part)
    n = frame[0].size
    outs = [Column.empty(t, n, with_valid=True) if e else Column(None, None, t, 0) for t, e in zip(types, evald)]
    fa, _fs = _colarray(frame)
    structs = []
    arr = (C.POINTER(GdfColumn) * max(1, len(outs)))()
    for i, c in enumerate(outs):
        s = c.to_c() if c.data is not None else GdfColumn()
        structs.append(s)
        arr[i] = C.pointer(s)
    _check(lib().ral_execute_project_plan(fa, len(frame), query_part.encode(), arr, len(outs)))
    _sync_categories(frame, _fs)
    result = []
    for i, (c, s, e) in enumerate(zip(outs, structs, evald)):
        if e:
            c.sync_from_c(s)
            result.append(c)
        else:
            src = next(f for f in frame if f.data is not None and f.data.data_ptr() == s.data) \
                if s.data else frame[0]
            src.null_count = int(s.null_count)
            result.append(src)
    return result


def filter_project(frame: List[Column], filter_query_part: str, project_query_part: str) -> List[Column]:
    """LogicalProject over LogicalFilter, fused: returns the projected, filtered frame."""
    types, evald = project_output_types([c.dtype for c in frame], project_query_part)
    n = frame[0].size
    srcs = _passthrough_sources(frame, project_query_part)
    outs = []
    for i, (t, e) in enumerate(zip(types, evald)):
        with_valid = True if e else (srcs[i].valid is not None)
        outs.append(Column.empty(t, n, with_valid=with_valid))
    fa, _fs = _colarray(frame)
    oa, ostructs = _colarray(outs)
    n_out = C.c_int32(0)
    _check(lib().ral_filter_project(fa, len(frame), filter_query_part.encode(), project_query_part.encode(), oa,
                                    len(outs), C.byref(n_out)))
    _sync_categories(frame, _fs)
    for col, s in zip(outs, ostructs):
        col.sync_from_c(s)
    return outs


def _passthrough_sources(frame: List[Column], project_query_part: str) -> dict:
    """Frame column behind each pass-through projection ("$k")."""
    out = {}
    inner = project_query_part[project_query_part.find("(") + 1:project_query_part.rfind(")")]
    depth, start, parts = 0, 0, []
    for i, ch in enumerate(inner):
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif ch == "," and depth == 0:
            parts.append(inner[start:i])
            start = i + 1
    parts.append(inner[start:])
    for i, p in enumerate(parts):
        body = p.strip()
        body = body[body.find("=[") + 2:-1]
        if "(" not in body.replace("CAST(", "").replace("):BIGINT", ""):
            out[i] = frame[int(body.strip()[1:])]
    return out


def materialize_column(input_column: Column, row_indices: Column, with_valid: Optional[bool] = None) -> Column:
    """materialize_column (src/ColumnManipulation.cuh:16-18): gather by row index."""
    n = row_indices.size
    wv = (input_column.valid is not None) if with_valid is None else with_valid
    out = Column.empty(input_column.dtype, n, with_valid=wv)
    ic, oc, rc = input_column.to_c(), out.to_c(), row_indices.to_c()
    _check(lib().ral_materialize_column(C.byref(ic), C.byref(oc), C.byref(rc)))
    out.sync_from_c(oc)
    return out


def materialize_columns(input_columns: List[Column], row_indices: Column,
                        with_valid: Optional[Sequence[bool]] = None) -> List[Column]:
    """Every column gathered by one index column in one kernel (the per-column materialize_column
    loops of JoinOperator.cpp:130,135 and OrderBy.cpp:66)."""
    n = row_indices.size
    wv = [c.valid is not None for c in input_columns] if with_valid is None else list(with_valid)
    outs = [Column.empty(c.dtype, n, with_valid=w) for c, w in zip(input_columns, wv)]
    ia, _is = _colarray(input_columns)
    oa, os_ = _colarray(outs)
    rc = row_indices.to_c()
    _check(lib().ral_materialize_columns(C.cast(ia, C.c_void_p), C.cast(oa, C.c_void_p), len(outs), C.byref(rc)))
    for o, st in zip(outs, os_):
        o.sync_from_c(st)
    return outs


def _text_device(data):
    """A uint8 device tensor of the text (bytes are copied to the GPU)."""
    import torch
    if isinstance(data, (bytes, bytearray, memoryview)):
        b = bytes(data)
        t = torch.frombuffer(bytearray(b), dtype=torch.uint8) if b else torch.zeros(0, dtype=torch.uint8)
        return t.to("cuda")
    return data


def text_scan_rows(data, line_terminator: bytes = b"\n", skip_rows: int = 0) -> int:
    """Rows of a delimited text buffer: lines after the first skip_rows that are not blank."""
    t = _text_device(data)
    rows = C.c_int64(0)
    _check(lib().ral_text_scan_rows(C.c_void_p(t.data_ptr() if t.numel() else 0), t.numel(), line_terminator,
                                    skip_rows, C.byref(rows)))
    return rows.value


def text_scan_filter(data, file_dtypes, projections, filter_query_part: Optional[str] = None, delimiter: bytes = b"|",
                     line_terminator: bytes = b"\n", skip_rows: int = 0, capacity: Optional[int] = None,
                     from_host: bool = False) -> List[Column]:
    """BindableTableScan over delimited text (projects = projections) fused with its LogicalFilter
    (None: the scan alone): the kept rows of the projected columns, every column with a mask.
    from_host=True passes the text in host memory (ral_text_scan_filter_host: copied in pieces,
    each scanned while the next is copied); otherwise it is copied to the device first."""
    if from_host:
        import torch
        if isinstance(data, torch.Tensor):
            h = data
        else:
            b = bytes(data)
            h = torch.frombuffer(bytearray(b), dtype=torch.uint8) if b else torch.zeros(0, dtype=torch.uint8)
        if capacity is None:
            capacity = text_scan_rows(h.to("cuda"), line_terminator, skip_rows)
        t, fn = h, lib().ral_text_scan_filter_host
    else:
        t = _text_device(data)
        if capacity is None:
            capacity = text_scan_rows(t, line_terminator, skip_rows)
        fn = lib().ral_text_scan_filter
    outs = [Column.empty(file_dtypes[c], capacity, with_valid=True) for c in projections]
    oa, os_ = _colarray(outs)
    n = C.c_int32(0)
    fd, pr = _i32(file_dtypes), _i32(projections)
    _check(fn(C.c_void_p(t.data_ptr() if t.numel() else 0), t.numel(), delimiter, line_terminator, skip_rows, _p32(fd),
              len(fd), _p32(pr), len(pr), filter_query_part.encode() if filter_query_part else None,
              C.cast(oa, C.c_void_p), C.byref(n)))
    for o, st in zip(outs, os_):
        o.sync_from_c(st)
    return outs


def debug_text_scan_source(file_dtypes, projections, filter_query_part: Optional[str] = None, compile: bool = False):
    """Generated CUDA source (and NVRTC log when compile=True) of the text scan kernel; needs no GPU."""
    fd, pr = _i32(file_dtypes), _i32(projections)
    src = C.create_string_buffer(1 << 20)
    log = C.create_string_buffer(1 << 16)
    _check(lib().ral_debug_text_scan_source(_p32(fd), len(fd), _p32(pr), len(pr),
                                            filter_query_part.encode() if filter_query_part else None,
                                            1 if compile else 0, src, len(src), log, len(log)))
    return src.value.decode(), log.value.decode()


def parquet_schema(file: bytes):
    """(rows, [gdf dtype each leaf scans as, GDF_invalid where unsupported]) of a Parquet file."""
    buf = C.create_string_buffer(bytes(file), len(file))
    rows, ncols = C.c_int64(0), C.c_int32(0)
    dts = np.zeros(256, dtype=np.int32)
    _check(lib().ral_parquet_schema(buf, len(file), C.byref(rows), C.byref(ncols), _p32(dts), len(dts)))
    return rows.value, [int(x) for x in dts[:ncols.value]]


def parquet_scan_filter(file: bytes, projections, filter_query_part: Optional[str] = None,
                        page_locked: bool = False) -> List[Column]:
    """BindableTableScan over a Parquet file (host bytes; projections = leaf indices) followed by
    its LogicalFilter (None: the scan alone).  page_locked=True hands the library the file in
    page-locked memory, which its kernels read in place instead of copying the pages in."""
    rows, dts = parquet_schema(file)
    for c in projections:
        if 0 <= c < len(dts) and dts[c] == D.GDF_invalid:
            # the library refuses the leaf too; no out column of its type can be made here
            raise RalError(2, f"leaf {c}: only INT32 (DATE), INT64 (TIMESTAMP_MILLIS), FLOAT and DOUBLE columns are scanned")
    outs = [Column.empty(dts[c] if 0 <= c < len(dts) else D.GDF_INT32, rows, with_valid=True) for c in projections]
    oa, os_ = _colarray(outs)
    pr = _i32(projections)
    n = C.c_int32(0)
    if page_locked:
        import torch
        host = torch.frombuffer(bytearray(file), dtype=torch.uint8).pin_memory() if len(file) else None
        buf = C.c_void_p(host.data_ptr() if host is not None else 0)
    else:
        buf = C.create_string_buffer(bytes(file), len(file))
    _check(lib().ral_parquet_scan_filter(buf, len(file), _p32(pr), len(pr),
                                         filter_query_part.encode() if filter_query_part else None,
                                         C.cast(oa, C.c_void_p), C.byref(n)))
    for o, st in zip(outs, os_):
        o.sync_from_c(st)
    return outs


def apply_boolean_mask(stencil: Column) -> Column:
    """Indices (INT32 column) of the rows whose stencil is valid and nonzero, in row order."""
    out = Column.empty(D.GDF_INT32, stencil.size, with_valid=False)
    sc, oc = stencil.to_c(), out.to_c()
    n = C.c_int32(0)
    _check(lib().ral_apply_boolean_mask(C.byref(sc), C.byref(oc), C.byref(n)))
    out.sync_from_c(oc)
    return out


def add_expression_to_plan(expression: str, expression_position: int, num_outputs: int, num_inputs: int,
                           new_input_indices: Sequence[int]):
    """The register-program emitter (src/LogicalFilter.h:26-42); returns the op arrays."""
    cap = 1024
    l, r, o = (np.zeros(cap, dtype=np.int16) for _ in range(3))
    b, u = np.zeros(cap, dtype=np.int32), np.zeros(cap, dtype=np.int32)
    ls, rs = (GdfScalar * cap)(), (GdfScalar * cap)()
    nii = _i16(new_input_indices)
    n = C.c_int32(0)
    _check(lib().ral_add_expression_to_plan(expression.encode(), expression_position, num_outputs, num_inputs,
                                            _p16(nii), len(nii), _p16(l), _p16(r), _p16(o), _p32(b), _p32(u), ls, rs,
                                            C.byref(n), cap))
    k = n.value
    return dict(left=l[:k].tolist(), right=r[:k].tolist(), outputs=o[:k].tolist(), operators=b[:k].tolist(),
                unary_operators=u[:k].tolist(), left_scalars=[Scalar.from_c(ls[i]) for i in range(k)],
                right_scalars=[Scalar.from_c(rs[i]) for i in range(k)])


def get_output_type_expression(frame_dtypes: Sequence[int], expression: str) -> int:
    fd = _i32(frame_dtypes)
    out = C.c_int32(0)
    _check(lib().ral_get_output_type_expression(_p32(fd), len(fd), expression.encode(), C.byref(out)))
    return out.value


def debug_program_source(input_dtypes, input_nullable, output_dtypes, output_nullable, left, right, outputs,
                         final_positions, operators, unary_operators, left_scalars, right_scalars,
                         compile: bool = False) -> Tuple[str, str]:
    """Generated CUDA source (and NVRTC log when compile=True) of a program; needs no GPU."""
    idt, inl, odt, onl = _i32(input_dtypes), _i32(input_nullable), _i32(output_dtypes), _i32(output_nullable)
    l, r, o, f = _i16(left), _i16(right), _i16(outputs), _i16(final_positions)
    b, u = _i32(operators), _i32(unary_operators)
    ls = _scalars([_as_scalar(s) for s in left_scalars])
    rs = _scalars([_as_scalar(s) for s in right_scalars])
    src = C.create_string_buffer(1 << 20)
    log = C.create_string_buffer(1 << 16)
    _check(lib().ral_debug_program_source(_p32(idt), _p32(inl), len(idt), _p32(odt), _p32(onl), len(odt), _p16(l),
                                          _p16(r), _p16(o), len(l), _p16(f), _p32(b), _p32(u), ls, rs,
                                          1 if compile else 0, src, len(src), log, len(log)))
    return src.value.decode(), log.value.decode()


def debug_filter_source(frame_dtypes, frame_nullable, filter_query_part: str, project_query_part=None,
                        compile: bool = False):
    """Generated CUDA source (and NVRTC log when compile=True) of the fused filter kernel; needs no GPU."""
    fd, fn = _i32(frame_dtypes), _i32(frame_nullable)
    src = C.create_string_buffer(1 << 20)
    log = C.create_string_buffer(1 << 16)
    _check(lib().ral_debug_filter_source(_p32(fd), _p32(fn), len(fd), filter_query_part.encode(),
                                         project_query_part.encode() if project_query_part else None,
                                         1 if compile else 0, src, len(src), log, len(log)))
    return src.value.decode(), log.value.decode()


def process_aggregate(frame: List[Column], query_part: str) -> List[Scalar]:
    """process_aggregate without GROUP BY (src/operators/GroupBy.cpp:531-590): one Scalar per
    aggregation, its expression inputs evaluated and reduced in one kernel."""
    arr, _structs = _colarray(frame)
    cap = 256
    res = (GdfScalar * cap)()
    n = C.c_int32(0)
    _check(lib().ral_process_aggregate(C.cast(arr, C.c_void_p), len(frame), query_part.encode(), res, cap,
                                       C.byref(n)))
    _sync_categories(frame, _structs)
    return [Scalar.from_c(res[i]) for i in range(n.value)]


def debug_aggregate_source(frame_dtypes, frame_nullable, frame_null_counts, query_part: str,
                           compile: bool = False):
    """Generated CUDA source (and NVRTC log when compile=True) of a LogicalAggregate's fused kernel;
    needs no GPU."""
    fd, fn = _i32(frame_dtypes), _i32(frame_nullable)
    nc = np.ascontiguousarray(np.asarray(frame_null_counts, dtype=np.int64))
    src = C.create_string_buffer(1 << 20)
    log = C.create_string_buffer(1 << 16)
    _check(lib().ral_debug_aggregate_source(_p32(fd), _p32(fn), nc.ctypes.data, len(fd), query_part.encode(),
                                            1 if compile else 0, src, len(src), log, len(log)))
    return src.value.decode(), log.value.decode()


def filter_project_host(frame: List[Column], filter_query_part: str, project_query_part: Optional[str],
                        out_columns: List[Column], chunk_rows: int = 0) -> int:
    """The fused filter (+ projection) over host-memory columns (torch CPU tensors, pinned for
    overlap) into host-memory outputs, streamed through the GPU in row chunks; returns the kept row
    count (out columns' size and null_count are set)."""
    fa, fs = _colarray(frame)
    oa, os_ = _colarray(out_columns)
    n = C.c_int32(0)
    _check(lib().ral_filter_project_host(C.cast(fa, C.c_void_p), len(frame), filter_query_part.encode(),
                                         project_query_part.encode() if project_query_part else None,
                                         C.cast(oa, C.c_void_p), len(out_columns), C.byref(n), int(chunk_rows)))
    for c, st in zip(out_columns, os_):
        c.sync_from_c(st)
    return n.value


def call_timing(enable: bool = True, reset: bool = False) -> dict:
    """Mean per-call breakdown (microseconds) of the synchronous filter entry points since the last
    reset: host preparation, enqueue, wait for completion and kernel device time."""
    calls = C.c_int64(0)
    us = (C.c_double * 4)()
    _check(lib().ral_debug_call_timing(1 if enable else 0, 1 if reset else 0, C.byref(calls), us))
    return {"calls": calls.value, "host_prepare_us": us[0], "enqueue_us": us[1], "wait_us": us[2],
            "kernel_device_us": us[3]}


def filter_grid_launches() -> int:
    """Fused filter launches that ran in grid mode (one grid barrier in place of the look-back)."""
    v = C.c_int64(0)
    _check(lib().ral_debug_filter_grid_launches(C.byref(v)))
    return v.value


class Category:
    """A string-category dictionary (ral_category): its distinct strings in byte order; a column's
    codes are their ranks.  Owned by the caller; dictionaries the library creates when a literal is
    missing are adopted with Category.adopt."""

    def __init__(self, handle: int):
        self.handle = int(handle)

    @staticmethod
    def create(strings: Sequence[str]) -> Tuple["Category", np.ndarray]:
        n = len(strings)
        enc = [s.encode() for s in strings]
        arr = (C.c_char_p * max(1, n))(*enc)
        codes = np.zeros(max(1, n), dtype=np.int32)
        h = C.c_void_p()
        _check(lib().ral_category_create(arr, n, C.byref(h), codes.ctypes.data_as(I32P)))
        return Category(h.value), codes[:n]

    @staticmethod
    def adopt(handle: int) -> "Category":
        return Category(handle)

    def size(self) -> int:
        n = C.c_int64(0)
        _check(lib().ral_category_size(C.c_void_p(self.handle), C.byref(n)))
        return n.value

    def get_value(self, s: str) -> int:
        code = C.c_int32(0)
        _check(lib().ral_category_get_value(C.c_void_p(self.handle), s.encode(), C.byref(code)))
        return code.value

    def keys(self) -> List[str]:
        out = []
        buf = C.create_string_buffer(1 << 12)
        ln = C.c_int64(0)
        for k in range(self.size()):
            _check(lib().ral_category_key(C.c_void_p(self.handle), k, buf, len(buf), C.byref(ln)))
            out.append(buf.raw[:ln.value].decode())
        return out

    def destroy(self) -> None:
        if self.handle:
            lib().ral_category_destroy(C.c_void_p(self.handle))
            self.handle = 0


def category_column(strings: Sequence[str], valids=None, device="cuda") -> Tuple[Column, Category]:
    """A GDF_STRING_CATEGORY column of the given strings (codes on the device, dictionary attached)."""
    cat, codes = Category.create(strings)
    col = Column.from_numpy(codes, D.GDF_STRING_CATEGORY, valids, device=device)
    col.category = cat.handle
    return col, cat


def decode_category(col: Column) -> List[Optional[str]]:
    """The strings of a category column's rows (None where null)."""
    keys = Category(col.category).keys()
    codes = col.to_numpy()
    vb = col.valid_bools()
    return [keys[c] if v else None for c, v in zip(codes, vb)]


def kernel_launches() -> int:
    return int(lib().ral_kernel_launches())


def jit_stats() -> dict:
    a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
    lib().ral_jit_stats(C.byref(a), C.byref(b), C.byref(c), C.byref(d))
    return dict(compiles=a.value, disk_hits=b.value, memory_hits=c.value, compile_ms=d.value)


def _stream_handle(stream) -> int:
    import torch
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def parse_project_plan(frame_dtypes: Sequence[int], query_part: str) -> dict:
    """parse_project_plan (src/CalciteInterpreter.cpp:123-309): the register program of a LogicalProject.

    Returns the frame columns the program reads (dense input order), the dtype of each evaluated
    expression and the op arrays (final positions are output registers n_in + k)."""
    fd = _i32(frame_dtypes)
    cap_ops, cap_cols = 4096, 1024
    nin, nev, nops = C.c_int32(0), C.c_int32(0), C.c_int32(0)
    inc = np.zeros(cap_cols, dtype=np.int32)
    edt = np.zeros(cap_cols, dtype=np.int32)
    l, r, o, f = (np.zeros(cap_ops, dtype=np.int16) for _ in range(4))
    b, u = np.zeros(cap_ops, dtype=np.int32), np.zeros(cap_ops, dtype=np.int32)
    ls, rs = (GdfScalar * cap_ops)(), (GdfScalar * cap_ops)()
    _check(lib().ral_parse_project_plan(_p32(fd), len(fd), query_part.encode(), cap_ops, cap_cols, C.byref(nin),
                                        _p32(inc), C.byref(nev), _p32(edt), C.byref(nops), _p16(l), _p16(r),
                                        _p16(o), _p16(f), _p32(b), _p32(u), ls, rs))
    k = nops.value
    return dict(input_columns=inc[:nin.value].tolist(), evaluated_dtypes=edt[:nev.value].tolist(),
                left=l[:k].tolist(), right=r[:k].tolist(), outputs=o[:k].tolist(),
                final_output_positions=f[:nev.value].tolist(), operators=b[:k].tolist(),
                unary_operators=u[:k].tolist(), left_scalars=[Scalar.from_c(ls[i]) for i in range(k)],
                right_scalars=[Scalar.from_c(rs[i]) for i in range(k)])


class Batch:
    """Many register programs run by one persistent kernel, replayed as a CUDA graph.

    add() takes perform_operation's arguments; the column descriptors are copied, so the
    buffers must stay allocated (and in place) for the life of the batch.  run() evaluates
    every program once, asynchronously on the given stream."""

    def __init__(self):
        h = C.c_void_p()
        _check(lib().ral_batch_create(C.byref(h)))
        self._h = h
        self._keep = []

    def add(self, output_columns: List[Column], input_columns: List[Column], left_inputs, right_inputs, outputs,
            final_output_positions, operators, unary_operators, left_scalars, right_scalars) -> int:
        oa, os_ = _colarray(output_columns)
        ia, is_ = _colarray(input_columns)
        l, r, o, f = _i16(left_inputs), _i16(right_inputs), _i16(outputs), _i16(final_output_positions)
        b, u = _i32(operators), _i32(unary_operators)
        ls = _scalars([_as_scalar(s) for s in left_scalars])
        rs = _scalars([_as_scalar(s) for s in right_scalars])
        idx = C.c_int32(-1)
        _check(lib().ral_batch_add(self._h, oa, len(output_columns), ia, len(input_columns), _p16(l), _p16(r),
                                   _p16(o), len(l), _p16(f), _p32(b), _p32(u), ls, rs, C.byref(idx)))
        self._keep.append((list(output_columns), list(input_columns)))
        return idx.value

    def prepare(self) -> None:
        _check(lib().ral_batch_prepare(self._h))

    def run(self, stream=None, use_graph: bool = True) -> None:
        _check(lib().ral_batch_run(self._h, C.c_void_p(_stream_handle(stream)), 1 if use_graph else 0))

    def info(self) -> dict:
        n, rows, items = C.c_int32(0), C.c_int64(0), C.c_int64(0)
        _check(lib().ral_batch_info(self._h, C.byref(n), C.byref(rows), C.byref(items)))
        regs, grid, per_sm = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        _check(lib().ral_batch_kernel_info(self._h, C.byref(regs), C.byref(grid), C.byref(per_sm)))
        return dict(programs=n.value, rows=rows.value, work_items=items.value, registers=regs.value,
                    grid=grid.value, blocks_per_sm=per_sm.value)

    def debug_source(self, compile: bool = False) -> Tuple[str, str]:
        src = C.create_string_buffer(1 << 24)
        log = C.create_string_buffer(1 << 16)
        _check(lib().ral_batch_debug_source(self._h, 1 if compile else 0, src, len(src), log, len(log)))
        return src.value.decode(), log.value.decode()

    def close(self) -> None:
        if self._h:
            lib().ral_batch_destroy(self._h)
            self._h = None
            self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_tune_key(output_columns: List[Column], input_columns: List[Column], left_inputs, right_inputs, outputs,
                   final_output_positions, operators, unary_operators, left_scalars, right_scalars) -> str:
    """The autotuner's table key of a program (dtype mix and program length)."""
    oa, _os = _colarray(output_columns)
    ia, _is = _colarray(input_columns)
    l, r, o, f = _i16(left_inputs), _i16(right_inputs), _i16(outputs), _i16(final_output_positions)
    b, u = _i32(operators), _i32(unary_operators)
    ls = _scalars([_as_scalar(s) for s in left_scalars])
    rs = _scalars([_as_scalar(s) for s in right_scalars])
    key = C.create_string_buffer(256)
    _check(lib().ral_batch_tune_key(oa, len(output_columns), ia, len(input_columns), _p16(l), _p16(r), _p16(o),
                                    len(l), _p16(f), _p32(b), _p32(u), ls, rs, key, len(key)))
    return key.value.decode()


def autotune_program(output_columns: List[Column], input_columns: List[Column], left_inputs, right_inputs, outputs,
                     final_output_positions, operators, unary_operators, left_scalars,
                     right_scalars) -> Tuple[int, int, bool, float]:
    """Times the program as a one-program batch at each candidate tile shape and records the
    best in the autotuner's table (used by batches); returns (slices, unroll, integer-pipe double
    operations, ms per launch)."""
    oa, _os = _colarray(output_columns)
    ia, _is = _colarray(input_columns)
    l, r, o, f = _i16(left_inputs), _i16(right_inputs), _i16(outputs), _i16(final_output_positions)
    b, u = _i32(operators), _i32(unary_operators)
    ls = _scalars([_as_scalar(s) for s in left_scalars])
    rs = _scalars([_as_scalar(s) for s in right_scalars])
    J, U, S, ms = C.c_int32(0), C.c_int32(0), C.c_int32(0), C.c_double(0)
    _check(lib().ral_autotune_program(oa, len(output_columns), ia, len(input_columns), _p16(l), _p16(r), _p16(o),
                                      len(l), _p16(f), _p32(b), _p32(u), ls, rs, C.byref(J), C.byref(U), C.byref(S),
                                      C.byref(ms)))
    return J.value, U.value, bool(S.value), ms.value


class Server:
    """Served execution: resident tables, prepared filter + project queries, requests run with
    continuous batching by a scheduler thread in the library (include/ral/ral_c.h)."""

    def __init__(self, budget_bytes: int = 120 << 30, max_waves: int = 2, max_wave_requests: int = 1024,
                 wave_rows: int = 0):
        h = C.c_void_p()
        _check(lib().ral_server_create(int(budget_bytes), max_waves, max_wave_requests, int(wave_rows), C.byref(h)))
        self._h = h
        self._tables = []

    def add_table(self, columns: List[Column]) -> int:
        arr, structs = _colarray(columns)
        tid = C.c_int32(-1)
        _check(lib().ral_server_add_table(self._h, arr, len(columns), C.byref(tid)))
        self._tables.append(list(columns))   # the server reads these buffers: keep them alive
        return tid.value

    def add_query(self, table_id: int, filter_query_part: str, project_query_part: str) -> int:
        qid = C.c_int32(-1)
        _check(lib().ral_server_add_query(self._h, table_id, filter_query_part.encode(), project_query_part.encode(),
                                          C.byref(qid)))
        return qid.value

    def query_outputs(self, query_id: int) -> Tuple[List[int], List[bool]]:
        cap = 64
        dt = np.zeros(cap, dtype=np.int32)
        hv = np.zeros(cap, dtype=np.int32)
        n = C.c_int32(0)
        _check(lib().ral_server_query_outputs(self._h, query_id, _p32(dt), _p32(hv), cap, C.byref(n)))
        return [int(x) for x in dt[:n.value]], [bool(x) for x in hv[:n.value]]

    def start(self) -> None:
        _check(lib().ral_server_start(self._h))

    def debug_compile(self) -> str:
        """Compiles every query's chunk function and links the dispatcher (no GPU needed)."""
        log = C.create_string_buffer(1 << 20)
        _check(lib().ral_server_debug_compile(self._h, log, len(log)))
        return log.value.decode()

    def submit(self, query_id: int, keep: bool = False) -> int:
        rid = C.c_int64(0)
        _check(lib().ral_server_submit(self._h, query_id, 1 if keep else 0, C.byref(rid)))
        return rid.value

    def wait(self, request_id: int, timeout_s: float = 120.0) -> Tuple[int, float]:
        rows, lat = C.c_int64(0), C.c_double(0)
        _check(lib().ral_server_wait(self._h, request_id, timeout_s, C.byref(rows), C.byref(lat)))
        return rows.value, lat.value

    def release(self, request_id: int) -> None:
        """Forgets a finished request (and frees its outputs if they were kept)."""
        _check(lib().ral_server_release(self._h, request_id))

    def result(self, request_id: int, query_id: int, release: bool = True) -> List[Column]:
        """Copies of a kept request's outputs (the server's buffers are released afterwards)."""
        dts, hv = self.query_outputs(query_id)
        rows = C.c_int64(0)
        _check(lib().ral_server_wait(self._h, request_id, 600.0, C.byref(rows), None))
        out = [Column.empty(dt, int(rows.value), with_valid=v) for dt, v in zip(dts, hv)]
        arr, structs = _colarray(out)
        _check(lib().ral_server_copy_result(self._h, request_id, arr, len(out)))
        for col, st in zip(out, structs):
            col.sync_from_c(st)
        if release:
            _check(lib().ral_server_release(self._h, request_id))
        return out

    def run_trace(self, queries, arrival_s) -> Tuple[np.ndarray, np.ndarray, float]:
        q = _i32(queries)
        a = np.ascontiguousarray(np.asarray(arrival_s, dtype=np.float64))
        lat = np.zeros(len(q), dtype=np.float64)
        rows = np.zeros(len(q), dtype=np.int64)
        mk = C.c_double(0)
        _check(lib().ral_server_run_trace(self._h, len(q), _p32(q), a.ctypes.data_as(C.POINTER(C.c_double)),
                                          lat.ctypes.data_as(C.POINTER(C.c_double)),
                                          rows.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(mk)))
        return lat, rows, mk.value

    def stats(self) -> dict:
        st = (C.c_int64 * 6)()
        _check(lib().ral_server_stats(self._h, st))
        solo, qs, rs = C.c_int64(0), C.c_double(0), C.c_double(0)
        _check(lib().ral_server_debug_stats(self._h, C.byref(solo), C.byref(qs), C.byref(rs)))
        return dict(submitted=st[0], completed=st[1], waves=st[2], max_wave_requests=st[3], peak_reserved=st[4],
                    busy_s=st[5] / 1e6, solo=solo.value, queue_s=qs.value, run_s=rs.value)

    def close(self) -> None:
        if self._h:
            lib().ral_server_destroy(self._h)
            self._h = None
            self._tables = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SOFTFP_OPS = ["div", "floor", "ceil", "compare", "i2d", "d2i", "f2d", "d2f", "is_zero", "fabs", "div64", "sincos"]


def softfp_selftest(n: int = 1 << 24, seed: int = 1) -> dict:
    """Runs the device self-test of the integer-pipe double operations; returns
    {op: (mismatches, first operand bits)}."""
    cnt = (C.c_int64 * 16)()
    first = (C.c_uint64 * 32)()
    _check(lib().ral_softfp_selftest(n, seed, cnt, first))
    return {op: (int(cnt[i]), (int(first[2 * i]), int(first[2 * i + 1]))) for i, op in enumerate(SOFTFP_OPS)}


def debug_lookback_timeout(n_rows: int = 3 * 4096) -> Tuple[int, int]:
    """Runs a compaction whose first tile is never taken; returns (status of that run, kept rows of
    a normal run right after)."""
    st, kept = C.c_int32(0), C.c_int64(0)
    _check(lib().ral_debug_lookback_timeout(n_rows, C.byref(st), C.byref(kept)))
    return st.value, kept.value
