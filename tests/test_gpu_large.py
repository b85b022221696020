"""Parity at scale: the fused filter kernels and the fused projection over tens to hundreds of
millions of rows, every output row compared bit for bit with the oracle.

These sizes exercise what small cases cannot: int32 row counts (gdf_size_type) near their range,
thousands of 1024-row chunk tickets and look-back steps, output validity words written at large bit
offsets, and columns whose byte size exceeds 2^31.  The check is the benchmark's chunked checker
(bench.parity_check): the oracle runs over row chunks on all host threads and each chunk's kept rows
are compared at their running output offset.
"""
import pytest

import bench

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def _run(ctx):
    import torch
    ctx["step"](torch.cuda.current_stream())
    torch.cuda.synchronize()


@pytest.mark.parametrize("null_rate", [None, 0.05])
def test_filter_gather_60M_rows(null_rate):
    ctx = bench.filter_setup("filter_gather", 60_000_003, 0.5, "cuda", null_rate=null_rate)
    _run(ctx)
    res = bench.parity_check("filter_gather", ctx, 0.5)
    assert res["mismatches"] == 0, res
    keep = 0.5 * (1.0 - (null_rate or 0.0))       # a null predicate drops its row
    assert abs(res["rows_out"] / res["rows"] - keep) < 0.01


@pytest.mark.parametrize("sel", [0.5, 0.99])
def test_filter_project_60M_rows(sel):
    ctx = bench.filter_setup("filter_project", 60_000_007, sel, "cuda")
    _run(ctx)
    res = bench.parity_check("filter_project", ctx, sel)
    assert res["mismatches"] == 0, res


def test_filter_gather_300M_rows_columns_above_2GiB():
    """300M rows: the int64 and float64 columns hold 2.4 GB each, so byte offsets pass 2^31."""
    ctx = bench.filter_setup("filter_gather", 300_000_001, 0.01, "cuda")
    _run(ctx)
    res = bench.parity_check("filter_gather", ctx, 0.01)
    assert res["mismatches"] == 0, res


def test_fused_projection_60M_rows():
    ctx = bench.fused_project_setup(60_000_011, "cuda")
    _run(ctx)
    res = bench.parity_check("fused_project", ctx, 0.5)
    assert res["mismatches"] == 0, res
