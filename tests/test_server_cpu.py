"""Served execution, host side: the workload plans, and every query's chunk function compiles
and links into the dispatcher (no GPU: the tables are host buffers that are never read)."""
import re

import numpy as np
import pytest

import ralgpu
from ralgpu import workloads as W


def _server_with_queries(n_tables, n_queries, seed=20261203, budget=120 << 30):
    tabs = W.served_tables(n_tables, seed=seed)
    qs = W.served_queries(tabs, n_queries, seed=seed)
    srv = ralgpu.Server(budget_bytes=budget)
    tids = []
    for t in tabs:
        cols = [ralgpu.Column.empty(dt, 1000, with_valid=True, device="cpu") for dt in t.dtypes]
        for c in cols:
            c.null_count = 1
        tids.append(srv.add_table(cols))
    qids = [srv.add_query(tids[q.table], q.filter, q.project) for q in qs]
    return srv, tabs, qs, qids


def test_served_workload_shapes():
    tabs = W.served_tables()
    assert len(tabs) == 24 and all(1e4 <= t.rows <= 1e8 for t in tabs)
    assert all(4 <= len(t.dtypes) <= 8 for t in tabs)
    qs = W.served_queries(tabs)
    assert all(4 <= q.n_ops <= 32 for q in qs)
    q, a = W.served_trace(5000, 200.0, len(qs))
    assert a[0] == 0.0 and np.all(np.diff(a) >= 0)
    assert abs(len(a) / a[-1] - 200.0) < 20.0    # Poisson at the requested rate
    assert q.min() >= 0 and q.max() < len(qs)


def test_every_query_plans_with_the_projection_it_names():
    srv, tabs, qs, qids = _server_with_queries(24, 96)
    for q, qid in zip(qs, qids):
        dts, hv = srv.query_outputs(qid)
        n_proj = q.project.count("=[")
        assert len(dts) == n_proj
        # evaluated expressions carry a mask; a pass-through column carries its column's mask
        assert all(hv)
    srv.close()


def test_query_chunk_functions_compile_and_link(tmp_path, monkeypatch):
    monkeypatch.setenv("RAL_JIT_CACHE_DIR", str(tmp_path))
    srv, tabs, qs, qids = _server_with_queries(6, 12)
    log = srv.debug_compile()
    frames = [int(m) for m in re.findall(r"(\d+) bytes stack frame", log)]
    assert frames and max(frames) < 2048
    srv.close()


def test_queries_with_identical_code_share_one_item_function(tmp_path, monkeypatch):
    """The same filter and projection over tables with the same column types generate one item
    function; it is linked once (a second copy is a duplicate symbol to the linker)."""
    monkeypatch.setenv("RAL_JIT_CACHE_DIR", str(tmp_path))
    D = ralgpu.dtypes
    srv = ralgpu.Server(budget_bytes=1 << 30)
    tids = [srv.add_table([ralgpu.Column.empty(D.GDF_INT32, n, with_valid=True, device="cpu"),
                           ralgpu.Column.empty(D.GDF_FLOAT64, n, with_valid=False, device="cpu")])
            for n in (0, 1, 1000)]
    fq, pq = "LogicalFilter(condition=[>($0, 5)])", "LogicalProject(x=[*($1, 2)], y=[$0])"
    for t in tids:
        srv.add_query(t, fq, pq)
        srv.add_query(t, fq, pq)
    srv.add_query(tids[1], "LogicalFilter(condition=[<($0, 5)])", pq)
    log = srv.debug_compile()
    assert "Multiple definition" not in log
    srv.close()


def test_budget_rejects_a_query_whose_request_cannot_fit():
    tabs = W.served_tables(2, seed=5)
    n = 100_000
    table_bytes = sum(n * ralgpu.dtypes.WIDTH[dt] + ralgpu.valid_alloc_size(n) for dt in tabs[0].dtypes)
    srv = ralgpu.Server(budget_bytes=table_bytes + (100 << 10))
    cols = [ralgpu.Column.empty(dt, n, with_valid=True, device="cpu") for dt in tabs[0].dtypes]
    tid = srv.add_table(cols)
    with pytest.raises(ralgpu.RalError, match="budget"):
        srv.add_query(tid, "LogicalFilter(condition=[<($0, 5)])",
                      "LogicalProject(a=[$0], b=[$1], c=[$2], d=[$3])")
    srv.close()
