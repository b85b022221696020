"""CPU ORACLE for the expression path (test infrastructure only).

The tests, the smoke check and the benchmark's CPU-baseline leg use this
package to compute expected results; the library under test never imports it.

* ``ral_oracle.cpp`` restates the reference Interpreter VM
  (src/Interpreter/interpreter_ops.cuh) row by row and the filter's mask and
  gather (src/CalciteInterpreter.cpp:509-573, src/ColumnManipulation.cu:26-150).
* ``frontend.py`` restates the RexNode text front end
  (src/CalciteExpressionParsing.cpp, src/LogicalFilter.cpp).

Parity is pinned by the reference's own known-answer tests, restated in
tests/golden/reference_kats.py (see tests/test_oracle_golden.py).
"""
from __future__ import annotations

import ctypes
import struct
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import frontend as fe
from .build import build as _build

_lib = None

NP_DTYPE = {
    fe.GDF_INT8: np.int8, fe.GDF_BOOL8: np.int8, fe.GDF_INT16: np.int16, fe.GDF_INT32: np.int32,
    fe.GDF_DATE32: np.int32, fe.GDF_STRING_CATEGORY: np.int32, fe.GDF_INT64: np.int64,
    fe.GDF_DATE64: np.int64, fe.GDF_TIMESTAMP: np.int64, fe.GDF_FLOAT32: np.float32,
    fe.GDF_FLOAT64: np.float64,
}


class _InCol(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("valid", ctypes.c_void_p), ("dtype", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("null_count", ctypes.c_int64)]


class _OutCol(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("valid", ctypes.c_void_p), ("dtype", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


class _Scalar(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int32), ("is_valid", ctypes.c_int32), ("bits", ctypes.c_uint64)]


def lib():
    global _lib
    if _lib is None:
        path = _build()
        L = ctypes.CDLL(path)
        L.oracle_perform_operation.restype = ctypes.c_int
        L.oracle_perform_operation.argtypes = [
            ctypes.c_int64, ctypes.POINTER(_InCol), ctypes.c_int, ctypes.POINTER(_OutCol), ctypes.c_int,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(_Scalar), ctypes.POINTER(_Scalar),
            ctypes.c_int, ctypes.c_int]
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_apply_boolean_mask.restype = ctypes.c_int64
        L.oracle_apply_boolean_mask.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_materialize_column.restype = ctypes.c_int
        L.oracle_materialize_column.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.POINTER(ctypes.c_int64)]
        L.oracle_infer_types.restype = ctypes.c_int
        L.oracle_force_valid_flags.restype = ctypes.c_int
        L.oracle_div_by_zero_events.restype = ctypes.c_longlong
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def valid_alloc_size(n: int) -> int:
    return ((n + 7) // 8 + 63) // 64 * 64


def pack_valid(bools: Sequence[bool] | np.ndarray, n: Optional[int] = None) -> np.ndarray:
    """LSB-first bitmask padded to 64 bytes; bits past n are 0."""
    b = np.asarray(bools, dtype=bool)
    n = len(b) if n is None else n
    out = np.zeros(valid_alloc_size(n), dtype=np.uint8)
    packed = np.packbits(b[:n], bitorder="little")
    out[:len(packed)] = packed
    return out


def unpack_valid(valid: Optional[np.ndarray], n: int) -> np.ndarray:
    if valid is None:
        return np.ones(n, dtype=bool)
    return np.unpackbits(valid, bitorder="little")[:n].astype(bool)


@dataclass
class OColumn:
    data: np.ndarray
    valid: Optional[np.ndarray]
    dtype: int
    null_count: int = 0
    category: Optional[list] = None   # GDF_STRING_CATEGORY: the dictionary, strings as bytes, sorted

    @property
    def size(self) -> int:
        return int(self.data.shape[0])

    def valid_bools(self) -> np.ndarray:
        return unpack_valid(self.valid, self.size)


def make_column(values, dtype: int, valids=None, null_count: Optional[int] = None) -> OColumn:
    data = np.ascontiguousarray(np.asarray(values).astype(NP_DTYPE[dtype]))
    if valids is None:
        return OColumn(data, None, dtype, 0)
    vb = np.asarray(valids, dtype=bool)
    nc = int((~vb).sum()) if null_count is None else null_count
    return OColumn(data, pack_valid(vb), dtype, nc)


def alloc_column(dtype: int, n: int, with_valid: bool = True) -> OColumn:
    """Like create_gdf_column: zeroed data, valid memset to 0xFF, null_count 0."""
    data = np.zeros(n, dtype=NP_DTYPE[dtype])
    valid = np.full(valid_alloc_size(n), 0xFF, dtype=np.uint8) if with_valid else None
    return OColumn(data, valid, dtype, 0)


def scalar_bits(s: fe.Scalar) -> int:
    t = s.dtype
    if t in (fe.GDF_FLOAT32,):
        raw = struct.pack("<f", float(s.value)) + b"\0" * 4
    elif t == fe.GDF_FLOAT64:
        raw = struct.pack("<d", float(s.value))
    elif t in (fe.GDF_INT8, fe.GDF_BOOL8):
        raw = struct.pack("<b", int(s.value)) + b"\0" * 7
    elif t == fe.GDF_INT16:
        raw = struct.pack("<h", int(s.value)) + b"\0" * 6
    elif t in (fe.GDF_INT32, fe.GDF_DATE32, fe.GDF_STRING_CATEGORY):
        raw = struct.pack("<i", int(s.value)) + b"\0" * 4
    else:
        raw = struct.pack("<q", int(s.value))
    return struct.unpack("<Q", raw)[0]


def _i16(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int16))


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def perform_operation(outputs: List[OColumn], inputs: List[OColumn], left, right, outs, final_positions,
                      operators, unary_operators, left_scalars: List[fe.Scalar],
                      right_scalars: List[fe.Scalar], nthreads: int = 1, float_literal_compat: bool = False,
                      n_rows: Optional[int] = None) -> None:
    L = lib()
    n_ops = len(left)
    n = inputs[0].size if n_rows is None else n_rows
    ic = (_InCol * max(1, len(inputs)))()
    for i, c in enumerate(inputs):
        ic[i].data = c.data.ctypes.data
        ic[i].valid = c.valid.ctypes.data if c.valid is not None else None
        ic[i].dtype = c.dtype
        ic[i].null_count = c.null_count
    oc = (_OutCol * max(1, len(outputs)))()
    for i, c in enumerate(outputs):
        oc[i].data = c.data.ctypes.data
        oc[i].valid = c.valid.ctypes.data if c.valid is not None else None
        oc[i].dtype = c.dtype
    ls = (_Scalar * max(1, n_ops))()
    rs = (_Scalar * max(1, n_ops))()
    for k in range(n_ops):
        for arr, s in ((ls, left_scalars[k]), (rs, right_scalars[k])):
            arr[k].dtype = s.dtype
            arr[k].is_valid = 1 if s.is_valid else 0
            arr[k].bits = scalar_bits(s)
    a_l, a_r, a_o, a_f = _i16(left), _i16(right), _i16(outs), _i16(final_positions)
    a_b, a_u = _i32(operators), _i32(unary_operators)
    rc = L.oracle_perform_operation(n, ic, len(inputs), oc, len(outputs), a_l.ctypes.data, a_r.ctypes.data,
                                    a_o.ctypes.data, n_ops, a_f.ctypes.data, a_b.ctypes.data, a_u.ctypes.data,
                                    ls, rs, nthreads, 1 if float_literal_compat else 0)
    if rc != 0:
        raise OracleError(L.oracle_last_error().decode())


def perform_plan(outputs: List[OColumn], inputs: List[OColumn], plan: fe.Plan, **kw) -> None:
    perform_operation(outputs, inputs, plan.left, plan.right, plan.outputs, plan.final_output_positions,
                      plan.operators, plan.unary_operators, plan.left_scalars, plan.right_scalars, **kw)


def make_category_column(strings, valids=None) -> OColumn:
    """A GDF_STRING_CATEGORY column: int32 codes = ranks of the strings in the sorted distinct set
    (NVCategory::create_from_array)."""
    keys = sorted(set(s.encode() for s in strings))
    rank = {k: i for i, k in enumerate(keys)}
    col = make_column([rank[s.encode()] for s in strings], fe.GDF_STRING_CATEGORY, valids)
    col.category = keys
    return col


class _Categories:
    """While planning over `frame`: a string literal compared with a category column is its code;
    a missing string is inserted in sorted position, and the column's codes at or above it move up
    by one (NVCategory::add_strings followed by the copy of the new values,
    src/LogicalFilter.cpp:161-193)."""

    def __init__(self, frame):
        self.frame = frame

    def resolve(self, col: int, s: str) -> int:
        import bisect
        c = self.frame[col]
        if c.dtype != fe.GDF_STRING_CATEGORY or c.category is None:
            raise OracleError("string literal compared with a column that is not a string category")
        key = s.encode()
        i = bisect.bisect_left(c.category, key)
        if i < len(c.category) and c.category[i] == key:
            return i
        c.category = c.category[:i] + [key] + c.category[i:]
        c.data[c.data >= i] += 1
        return i

    def sync(self, a: int, b: int) -> None:
        ca, cb = self.frame[a], self.frame[b]
        if a == b or ca.dtype != fe.GDF_STRING_CATEGORY or cb.dtype != fe.GDF_STRING_CATEGORY:
            return
        if ca.category == cb.category:
            return
        merged = sorted(set(ca.category) | set(cb.category))
        rank = {k: i for i, k in enumerate(merged)}
        for c in (ca, cb):
            table = np.array([rank[k] for k in c.category], dtype=np.int32)
            ok = (c.data >= 0) & (c.data < len(table))
            c.data[ok] = table[c.data[ok]]
            c.category = list(merged)

    def __enter__(self):
        self.prev = (fe.CATEGORY_RESOLVER, fe.CATEGORY_SYNC)
        fe.CATEGORY_RESOLVER = self.resolve
        fe.CATEGORY_SYNC = self.sync
        return self

    def __exit__(self, *a):
        fe.CATEGORY_RESOLVER, fe.CATEGORY_SYNC = self.prev


def decode_category(col: OColumn) -> list:
    vb = col.valid_bools()
    return [col.category[c].decode() if v else None for c, v in zip(col.data, vb)]


def evaluate_expression(frame: List[OColumn], expression: str, output: OColumn, **kw) -> OColumn:
    """Returns the output column (a clone of a frame column for the "$n" shortcut)."""
    with _Categories(frame):
        res = fe.plan_evaluate_expression(len(frame), expression)
    if res[0] == "clone":
        src = frame[res[1]]
        return OColumn(src.data.copy(), None if src.valid is None else src.valid.copy(), src.dtype,
                       src.null_count)
    _, plan, cols = res
    perform_plan([output], [frame[c] for c in cols], plan, **kw)
    return output


def update_null_count(col: OColumn) -> None:
    if col.size == 0 or col.valid is None:
        col.null_count = 0
    else:
        col.null_count = int(col.size - col.valid_bools().sum())


def apply_boolean_mask(stencil: OColumn) -> np.ndarray:
    if stencil.data.dtype.itemsize != 1:
        raise OracleError("stencil must be a one-byte column")
    n = stencil.size
    idx = np.zeros(max(n, 1), dtype=np.int32)
    k = lib().oracle_apply_boolean_mask(n, stencil.data.ctypes.data,
                                        stencil.valid.ctypes.data if stencil.valid is not None else None,
                                        idx.ctypes.data)
    return idx[:k].copy()


def materialize_column(col: OColumn, idx: np.ndarray) -> OColumn:
    n_out = len(idx)
    data = np.zeros(max(n_out, 1), dtype=col.data.dtype)
    valid = np.zeros(valid_alloc_size(n_out), dtype=np.uint8) if col.valid is not None else None
    nc = ctypes.c_int64(0)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    lib().oracle_materialize_column(col.data.ctypes.data, col.valid.ctypes.data if col.valid is not None else None,
                                    col.data.dtype.itemsize, idx.ctypes.data if n_out else None, n_out,
                                    data.ctypes.data, valid.ctypes.data if valid is not None else None,
                                    ctypes.byref(nc))
    return OColumn(data[:n_out], valid, col.dtype, int(nc.value), col.category)


def process_filter(frame: List[OColumn], query_part: str, **kw) -> List[OColumn]:
    """LogicalFilter: stencil -> boolean mask over the row indices -> gather every column."""
    n = frame[0].size
    if n == 0:
        return frame
    stencil = alloc_column(fe.GDF_INT8, n)
    cond = fe.get_condition_expression(query_part)
    stencil = evaluate_expression(frame, cond, stencil, **kw)
    idx = apply_boolean_mask(stencil)
    return [materialize_column(c, idx) for c in frame]


def filter_indices(frame: List[OColumn], query_part: str, **kw) -> np.ndarray:
    n = frame[0].size
    stencil = alloc_column(fe.GDF_INT8, n)
    stencil = evaluate_expression(frame, fe.get_condition_expression(query_part), stencil, **kw)
    return apply_boolean_mask(stencil)


def execute_project_plan(frame: List[OColumn], query_part: str, **kw) -> List[OColumn]:
    """LogicalProject: every evaluated expression in one program, pass-through columns shared."""
    with _Categories(frame):
        pp = fe.parse_project_plan([c.dtype for c in frame], query_part)
    n = frame[0].size
    outs = [alloc_column(t, n) for t in pp.output_types]
    if outs:
        perform_plan(outs, [frame[c] for c in pp.input_columns], pp.plan, **kw)
    result = []
    for kind, v in pp.columns:
        result.append(outs[v] if kind == "expr" else frame[v])
    for c in result:
        update_null_count(c)
    return result


# ---- aggregations without GROUP BY (src/operators/GroupBy.cpp) -----------------------------------

@dataclass
class AggResult:
    dtype: int
    is_valid: bool
    value: object = None        # int or float (the exactly rounded sum for a float SUM / AVG)
    float_sum_bound: float = 0.0  # float SUM / AVG: sum of |x|, for the error bound of any order


def process_aggregate(frame: List[OColumn], query_part: str, **kw) -> List[AggResult]:
    """process_aggregate without GROUP BY, as the reference runs it (GroupBy.cpp:531-590,
    compute_aggregations :298-345, aggregations_without_groupby :231-296): an input that contains
    an evaluation is evaluated into a column of its own (evaluate_expression, which leaves the
    column's null_count at 0, LogicalFilter.cpp:368); any other input is a frame column (get_index;
    COUNT() reads column 0).  The reduction (cudf::reduce, not vendored) consults the mask only
    when null_count > 0; SUM widens to INT64 / FLOAT64, MIN / MAX keep the input type with the
    numeric_limits max / lowest identities, AVG divides the sum by size - null_count, COUNT is
    size - null_count; an empty or all-null input gives a null (invalid) scalar.  A float SUM has
    no defined order in the reference: its value here is the exactly rounded sum (math.fsum)."""
    import math
    groups, aggs = fe.parse_aggregate(query_part)
    if groups:
        raise OracleError("GROUP BY aggregations are not restated")
    n = frame[0].size
    dtypes = [c.dtype for c in frame]
    out = []
    for name, op, expr in aggs:
        if fe.contains_evaluation(expr):
            t = fe.get_output_type_expression(dtypes, expr)
            col = evaluate_expression(frame, expr, alloc_column(t, n), **kw)
            col.null_count = 0
        else:
            col = frame[fe.get_index(expr)]
        out_t = fe.get_aggregation_output_type(col.dtype, op)
        count = col.size - col.null_count
        if op == fe.GDF_COUNT:
            out.append(AggResult(out_t, True, int(count)))
            continue
        if col.size == 0 or col.size <= col.null_count:
            out.append(AggResult(out_t, False))
            continue
        vals = col.data[col.valid_bools()] if (col.valid is not None and col.null_count > 0) else col.data
        flt = fe.is_type_float(col.dtype)
        if op in (fe.GDF_SUM, fe.GDF_AVG):
            if flt:
                v64 = vals.astype(np.float64)
                s = math.fsum(v64.tolist())
                bound = float(np.abs(v64).sum())
            else:
                s = int(vals.astype(np.int64).astype(np.uint64).sum(dtype=np.uint64).astype(np.int64))
                bound = 0.0
            if op == fe.GDF_SUM:
                out.append(AggResult(out_t, True, s, bound))
            else:
                out.append(AggResult(fe.GDF_FLOAT64, True, float(s) / float(count), bound / float(count)))
            continue
        info = np.finfo(vals.dtype) if flt else np.iinfo(vals.dtype)
        ident = info.max if op == fe.GDF_MIN else (info.min if not flt else -info.max)
        m = vals.min() if op == fe.GDF_MIN else vals.max()
        m = min(m, ident) if op == fe.GDF_MIN else max(m, ident)
        out.append(AggResult(out_t, True, float(m) if flt else int(m)))
    return out
