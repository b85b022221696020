"""ral_filter_project_host: the fused filter (and filter + project) over host-memory columns,
streamed through the GPU in row chunks, against the device entry points and the oracle.  Small
chunks make many chunks whose kept rows land at output offsets that are not multiples of 8 or 32,
so the merge of each chunk's first mask word with the rows before it is exercised."""
import numpy as np
import pytest
import torch

import oracle as O
import ralgpu as R
from ralgpu import dtypes as D
from ralgpu import workloads as W

from helpers import to_device, to_oracle

pytestmark = pytest.mark.gpu


def _host(col: R.Column) -> R.Column:
    return R.Column(col.data.cpu().pin_memory(), None if col.valid is None else col.valid.cpu().pin_memory(),
                    col.dtype, col.size, col.null_count, col.category)


def _host_out(dtype, n, with_valid):
    data = torch.empty(max(n, 1), dtype=D.torch_dtype(dtype)).pin_memory()
    valid = torch.full((R.valid_alloc_size(max(n, 1)),), 0xAB, dtype=torch.uint8).pin_memory() if with_valid else None
    return R.Column(data, valid, dtype, n)


def _compare(got, exp):
    assert got.size == exp.size
    gv = got.valid_bools() if got.valid is not None else None
    if gv is not None:
        np.testing.assert_array_equal(gv, exp.valid_bools())
        assert got.null_count == exp.null_count
    m = exp.valid_bools()
    g = got.data[:got.size].numpy()
    e = exp.to_numpy() if isinstance(exp, R.Column) else exp.data
    u = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[g.dtype.itemsize]
    np.testing.assert_array_equal(g.view(u)[m], np.asarray(e).astype(g.dtype).view(u)[m])


@pytest.mark.parametrize("chunk", [1024, 5120, 0])
@pytest.mark.parametrize("sel", [0.01, 0.37, 0.99])
def test_filter_project_from_host_buffers(chunk, sel):
    n = 200_003
    spec = W.fused_project_host(n, seed=int(sel * 100) + chunk)
    dev = to_device(spec)
    fq, pq = W.filter_project_filter(sel), W.FILTER_PROJECT_PROJECT
    exp = R.filter_project(dev, fq, pq)
    host = [_host(c) for c in dev]
    outs = [_host_out(c.dtype, n, True) for c in exp]
    k = R.filter_project_host(host, fq, pq, outs, chunk_rows=chunk)
    assert k == exp[0].size
    for g, e in zip(outs, exp):
        _compare(g, e)
    # and the oracle
    f = O.process_filter(to_oracle(spec), fq)
    for g, e in zip(outs, O.execute_project_plan(f, pq)):
        _compare(g, e)


@pytest.mark.parametrize("chunk", [1024, 0])
def test_filter_gather_from_host_buffers(chunk):
    n = 300_007
    spec = W.filter_gather_host(n, seed=3, null_rate=0.05)
    dev = to_device(spec)
    q = W.filter_gather_query(0.5)
    exp = R.process_filter(dev, q)
    host = [_host(c) for c in dev]
    outs = [_host_out(c.dtype, n, c.valid is not None) for c in dev]
    k = R.filter_project_host(host, q, None, outs, chunk_rows=chunk)
    assert k == exp[0].size
    for g, e in zip(outs, exp):
        _compare(g, e)


def test_host_filter_keeps_nothing_and_everything():
    n = 70_001
    spec = W.filter_gather_host(n, seed=4)
    host = [_host(c) for c in to_device(spec)]
    for q, want in (("LogicalFilter(condition=[<($0, 0)])", 0), ("LogicalFilter(condition=[>=($0, 0)])", n)):
        outs = [_host_out(c.dtype, n, c.valid is not None) for c in host]
        assert R.filter_project_host(host, q, None, outs, chunk_rows=2048) == want
