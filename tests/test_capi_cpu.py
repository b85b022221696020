"""The C-ABI library loads and exports every symbol include/ral/*.h declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

import ralgpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include", "ral")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ral_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_declared_symbols_nonempty():
    syms = declared_symbols()
    assert "ral_perform_operation" in syms
    assert "ral_process_filter" in syms
    assert len(syms) >= 12


@pytest.mark.parametrize("sym", declared_symbols())
def test_symbol_exported(sym):
    L = ralgpu.lib()
    assert hasattr(L, sym), f"{sym} declared in include/ral but not exported by libralgpu.so"


def test_version_and_error_string():
    assert "sm_103a" in ralgpu.version()
    assert isinstance(ralgpu.lib().ral_last_error(), bytes)


def test_invalid_program_rejected_without_gpu():
    """Validation happens on the host before any CUDA call."""
    from ralgpu.column import GdfColumn
    L = ralgpu.lib()
    col = GdfColumn()
    col.size = 4
    col.dtype = 4
    arr = (ctypes.POINTER(GdfColumn) * 1)(ctypes.pointer(col))
    rc = L.ral_perform_operation(arr, 1, arr, 0, None, None, None, 0, None, None, None, None, None, None, 0)
    assert rc == 1
    assert b"input" in L.ral_last_error()


def test_host_buffer_evaluation_checks_arguments_before_any_cuda_call():
    """ral_perform_operation_host validates columns and the program on the host; an empty frame
    returns at once with zero null counts."""
    import numpy as np
    from ralgpu import dtypes as D
    from ralgpu import workloads as W
    spec = W.fused_project_program()
    cols = [ralgpu.Column.from_numpy(np.zeros(8, dtype=np.int64 if t == D.GDF_INT64 else
                                              (np.float64 if t == D.GDF_FLOAT64 else np.int32)), t, None, device="cpu")
            for t in spec.input_dtypes]
    outs = [ralgpu.Column.empty(t, 8, device="cpu") for t in spec.output_dtypes]
    args = (spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops, spec.lscalars, spec.rscalars)
    short = ralgpu.Column.from_numpy(np.zeros(4, dtype=np.int32), D.GDF_INT32, None, device="cpu")
    with pytest.raises(ralgpu.RalError, match="differ in size"):
        ralgpu.perform_operation_host(outs, cols[:4] + [short], *args)
    with pytest.raises(ralgpu.RalError, match="shorter"):
        ralgpu.perform_operation_host([ralgpu.Column.empty(t, 2, device="cpu") for t in spec.output_dtypes], cols, *args)
    empty = [ralgpu.Column.from_numpy(np.zeros(0, dtype=c.to_numpy().dtype), c.dtype, None, device="cpu") for c in cols]
    eouts = [ralgpu.Column.empty(t, 0, device="cpu") for t in spec.output_dtypes]
    for c in eouts:
        c.null_count = 5
    ralgpu.perform_operation_host(eouts, empty, *args)
    assert all(c.null_count == 0 for c in eouts)


def test_materialize_columns_checks_arguments_before_any_cuda_call():
    """ral_materialize_columns rejects more than 64 columns, a floating-point index column, width
    mismatches and inputs of different sizes on the host; no columns is a no-op."""
    import numpy as np
    from ralgpu import dtypes as D
    from ralgpu.column import GdfColumn
    L = ralgpu.lib()
    keep = []

    def mk(t, n):
        c = ralgpu.Column.from_numpy(np.zeros(n, dtype=D.NP[t]), t, None, device="cpu")
        keep.append(c)
        return c.to_c()

    def call(ins, outs, idx):
        ia = (ctypes.POINTER(GdfColumn) * max(1, len(ins)))(*[ctypes.pointer(x) for x in ins])
        oa = (ctypes.POINTER(GdfColumn) * max(1, len(outs)))(*[ctypes.pointer(x) for x in outs])
        keep.extend([ia, oa])
        return L.ral_materialize_columns(ctypes.cast(ia, ctypes.c_void_p), ctypes.cast(oa, ctypes.c_void_p),
                                         len(ins), ctypes.byref(idx))

    idx = mk(D.GDF_INT32, 4)
    cols = [mk(D.GDF_INT32, 8) for _ in range(65)]
    assert call(cols, cols, idx) == 1 and b"columns" in L.ral_last_error()
    assert call(cols[:1], cols[:1], mk(D.GDF_FLOAT32, 4)) == 1 and b"row_indices" in L.ral_last_error()
    assert call([mk(D.GDF_INT32, 8), mk(D.GDF_INT64, 9)], [mk(D.GDF_INT32, 4), mk(D.GDF_INT64, 4)], idx) == 1
    assert b"differ in size" in L.ral_last_error()
    assert call([mk(D.GDF_INT32, 8)], [mk(D.GDF_INT64, 8)], idx) == 1 and b"width mismatch" in L.ral_last_error()
    assert call([], [], idx) == 0


def test_category_dictionary_api_needs_no_gpu():
    """ral_category: distinct strings sorted by byte value, codes are ranks, -1 for a missing string."""
    strings = ["pear", "apple", "Zebra", "apple", "é", "banana", ""]
    cat, codes = ralgpu.Category.create(strings)
    keys = cat.keys()
    assert keys == sorted(set(strings), key=lambda s: s.encode())
    assert [keys[c] for c in codes] == strings
    assert cat.get_value("banana") == keys.index("banana") and cat.get_value("kiwi") == -1
    assert cat.size() == len(set(strings))
    cat.destroy()
