"""ral_apply_boolean_mask_noalloc: the allocation-free compaction entry point.

Callers that cannot allocate device memory (a pool that owns the whole GPU, a
latency-critical path kept out of the driver's allocator) use this variant; its
scratch is a fixed array inside the library.  These tests call it through the C
ABI and check it against the allocating ral_apply_boolean_mask, twice in a row so
that a second call cannot see the first call's leftover tile states.  The file is
named to be collected last; it also passes when run alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import ralgpu as R
from ralgpu import dtypes as D
from ralgpu.column import GdfColumn

pytestmark = pytest.mark.gpu

MAX_ROWS = (256 * 1024 // 8 - 3) * 4096   # RAL_NOALLOC_MAX_ROWS in include/ral/ral_c.h


def _entry():
    f = R.lib().ral_apply_boolean_mask_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(GdfColumn), ctypes.POINTER(GdfColumn), ctypes.POINTER(ctypes.c_int32)]
    return f


def _noalloc(stencil: R.Column, out: R.Column = None) -> R.Column:
    if out is None:
        out = R.Column.empty(D.GDF_INT32, stencil.size, with_valid=False)
    sc, oc = stencil.to_c(), out.to_c()
    n = ctypes.c_int32(-1)
    rc = _entry()(ctypes.byref(sc), ctypes.byref(oc), ctypes.byref(n))
    assert rc == 0, R.lib().ral_last_error().decode()
    out.sync_from_c(oc)
    assert n.value == out.size
    return out


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    rng = np.random.default_rng(20261203)
    # the second call is smaller and sparser than the first: stale tile states from the
    # first call would corrupt it if the shared array were not cleared
    for n, keep_rate, null_rate in ((3_000_017, 0.9, 0.05), (1_000_003, 0.3, 0.2)):
        stencil = np.where(rng.random(n) < keep_rate, rng.integers(1, 4, n), 0).astype(np.int8)
        valid = rng.random(n) >= null_rate
        col = R.Column.from_numpy(stencil, D.GDF_INT8, valid)
        got = _noalloc(col)
        exp = R.apply_boolean_mask(col)
        assert got.size == exp.size
        np.testing.assert_array_equal(got.to_numpy(), exp.to_numpy())


def _cudart():
    """The CUDA runtime the library links (for the default memory pool's counters)."""
    import glob
    import os
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            pass
    for cand in glob.glob(os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so*")):
        return ctypes.CDLL(cand)
    pytest.skip("libcudart not found")


def test_noalloc_makes_no_device_allocation():
    """The property the entry point exists for: a warm call (and an empty one) leaves the device's
    free memory and its default memory pool's high-water mark where they were."""
    import torch
    rt = _cudart()
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), torch.cuda.current_device()) == 0
    USED_CURRENT, USED_HIGH = 7, 8          # cudaMemPoolAttrUsedMemCurrent / UsedMemHigh
    rng = np.random.default_rng(5)
    n = 2_000_003
    col = R.Column.from_numpy((rng.random(n) < 0.5).astype(np.int8), D.GDF_INT8, rng.random(n) >= 0.1)
    empty = R.Column.empty(D.GDF_INT8, 0, with_valid=False)
    # outputs made up front: only the calls themselves run between the two readings
    out = R.Column.empty(D.GDF_INT32, n, with_valid=False)
    out0 = R.Column.empty(D.GDF_INT32, 0, with_valid=False)
    _noalloc(col, out)                      # warm: module loaded, kernel resolved
    torch.cuda.synchronize()
    # resetting the high-water mark sets it to the pool memory in use now (other callers' blocks)
    zero = ctypes.c_uint64(0)
    assert rt.cudaMemPoolSetAttribute(pool, USED_HIGH, ctypes.byref(zero)) == 0
    used0 = ctypes.c_uint64(0)
    assert rt.cudaMemPoolGetAttribute(pool, USED_CURRENT, ctypes.byref(used0)) == 0
    free0, _ = torch.cuda.mem_get_info()
    got = _noalloc(col, out)
    assert _noalloc(empty, out0).size == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    high = ctypes.c_uint64(1)
    assert rt.cudaMemPoolGetAttribute(pool, USED_HIGH, ctypes.byref(high)) == 0
    assert high.value <= used0.value, "the call allocated from the default memory pool"
    assert free1 == free0, "device free memory changed across the call"
    assert got.size == R.apply_boolean_mask(col).size


def test_noalloc_rejects_stencils_beyond_the_limit():
    col = R.Column.empty(D.GDF_INT8, 64, with_valid=False)
    out = R.Column.empty(D.GDF_INT32, 64, with_valid=False)
    sc, oc = col.to_c(), out.to_c()
    sc.size = MAX_ROWS + 1           # rejected on the host, before any device access
    n = ctypes.c_int32(-1)
    rc = _entry()(ctypes.byref(sc), ctypes.byref(oc), ctypes.byref(n))
    assert rc == 1
    assert b"scratch limit" in R.lib().ral_last_error()
