"""ral_materialize_columns: every column of a frame gathered by one index column, against the
oracle's materialize_column (src/ColumnManipulation.cu:137-150) run column by column, and against
the library's own single-column ral_materialize_column.

Cases: element widths 1 / 2 / 4 / 8 (int8, bool8, int16, int32, date32, float32, int64, float64),
nullable and non-nullable sources, index columns of every integer width, random indices with
repetition (join-like), permutations (order-by), sorted indices (filter-like), negative indices
(rows left unwritten and null), row counts that are not multiples of 32 or of 128, an empty index
column, one column and the 64-column maximum.
"""
import numpy as np
import pytest

import oracle as O
import ralgpu as R
from ralgpu import dtypes as D

from helpers import to_device, to_oracle

pytestmark = pytest.mark.gpu

FRAME_DTYPES = [D.GDF_INT8, D.GDF_BOOL8, D.GDF_INT16, D.GDF_INT32, D.GDF_DATE32, D.GDF_FLOAT32, D.GDF_INT64,
                D.GDF_FLOAT64]
IDX_DTYPE = {1: D.GDF_INT8, 2: D.GDF_INT16, 4: D.GDF_INT32, 8: D.GDF_INT64}
IDX_NP = {1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}


def _frame(rng, n, dtypes, null_rate):
    spec = []
    for k, t in enumerate(dtypes):
        if t in (D.GDF_FLOAT32, D.GDF_FLOAT64):
            v = rng.standard_normal(n)
        elif t == D.GDF_BOOL8:
            v = rng.integers(0, 2, n)
        else:
            info = np.iinfo(D.NP[t])
            v = rng.integers(info.min, info.max, n, endpoint=True, dtype=np.int64)
        m = (rng.random(n) >= null_rate) if (null_rate and k % 2 == 0) else None
        spec.append((t, v, m))
    return spec


def _indices(rng, n_in, n_out, pattern, width):
    hi = min(n_in, np.iinfo(IDX_NP[width]).max + 1)
    if pattern == "random":
        idx = rng.integers(0, hi, n_out)
    elif pattern == "permutation":
        idx = rng.permutation(hi)[:n_out]
    elif pattern == "sorted":
        idx = np.sort(rng.integers(0, hi, n_out))
    else:  # with negatives: unwritten, null rows
        idx = rng.integers(0, hi, n_out)
        idx[rng.random(n_out) < 0.1] = -1
    return idx.astype(IDX_NP[width])


def _check(frame_spec, idx):
    n_out = len(idx)
    dev = to_device(frame_spec)
    ora = to_oracle(frame_spec)
    w = idx.dtype.itemsize
    ic = R.Column.from_numpy(idx, IDX_DTYPE[w])
    got = R.materialize_columns(dev, ic)
    keep = idx >= 0
    for c, (g, oc) in enumerate(zip(got, ora)):
        exp = O.materialize_column(oc, idx.astype(np.int32))
        assert g.size == n_out
        if oc.valid is not None:
            gv, ev = g.valid_bools(), exp.valid_bools()
            np.testing.assert_array_equal(gv, ev, err_msg=f"column {c}: validity")
            assert g.null_count == exp.null_count, (c, g.null_count, exp.null_count)
        else:
            assert g.valid is None and g.null_count == 0
        gd = g.to_numpy()
        ed = exp.data[:n_out]
        u = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[gd.dtype.itemsize]
        np.testing.assert_array_equal(gd.view(u)[keep], ed.astype(gd.dtype).view(u)[keep],
                                      err_msg=f"column {c}: data")
        # the single-column entry point gives the same bits
        single = R.materialize_column(dev[c], ic)
        np.testing.assert_array_equal(single.to_numpy().view(u)[keep], gd.view(u)[keep])
        if g.valid is not None:
            np.testing.assert_array_equal(single.valid_bools(), g.valid_bools())
            assert single.null_count == g.null_count


@pytest.mark.parametrize("width", [1, 2, 4, 8])
@pytest.mark.parametrize("pattern", ["random", "permutation", "sorted", "negatives"])
def test_gather_columns_matches_oracle(width, pattern):
    rng = np.random.default_rng(100 * width + len(pattern))
    n_in = 100_003
    n_out = 77_777 if pattern != "permutation" else min(n_in, np.iinfo(IDX_NP[width]).max + 1) - 5
    spec = _frame(rng, n_in, FRAME_DTYPES, 0.1)
    _check(spec, _indices(rng, n_in, n_out, pattern, width))


@pytest.mark.parametrize("n_out", [0, 1, 31, 32, 127, 128, 129, 4097])
def test_gather_columns_small_and_ragged(n_out):
    rng = np.random.default_rng(n_out)
    spec = _frame(rng, 5_000, FRAME_DTYPES, 0.2)
    _check(spec, _indices(rng, 5_000, n_out, "negatives", 4))


def test_gather_one_column_and_the_maximum():
    rng = np.random.default_rng(3)
    spec1 = _frame(rng, 10_000, [D.GDF_FLOAT64], 0.3)
    _check(spec1, _indices(rng, 10_000, 9_999, "random", 8))
    spec64 = _frame(rng, 20_000, [FRAME_DTYPES[k % len(FRAME_DTYPES)] for k in range(64)], 0.05)
    _check(spec64, _indices(rng, 20_000, 30_001, "random", 4))


def test_gather_columns_limits():
    rng = np.random.default_rng(4)
    spec = _frame(rng, 100, [D.GDF_INT32] * 65, 0.0)
    dev = to_device(spec)
    ic = R.Column.from_numpy(np.arange(10, dtype=np.int32), D.GDF_INT32)
    with pytest.raises(R.RalError):
        R.materialize_columns(dev, ic)
    assert R.materialize_columns([], ic) == []


def test_gather_columns_large_permutation():
    """An order-by-like permutation of 20M rows over six columns: every row compared."""
    import torch
    rng = np.random.default_rng(9)
    n = 20_000_003
    spec = _frame(rng, n, [D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64, D.GDF_DATE32, D.GDF_BOOL8], 0.05)
    idx = rng.permutation(n).astype(np.int32)
    dev = to_device(spec)
    got = R.materialize_columns(dev, R.Column.from_numpy(idx, D.GDF_INT32))
    torch.cuda.synchronize()
    for (t, v, m), g in zip(spec, got):
        exp = np.asarray(v).astype(D.NP[t])[idx]
        np.testing.assert_array_equal(g.to_numpy(), exp)
        if m is not None:
            np.testing.assert_array_equal(g.valid_bools(), np.asarray(m)[idx])
            assert g.null_count == int((~np.asarray(m)[idx]).sum())
