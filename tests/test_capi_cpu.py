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
