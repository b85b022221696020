"""Served execution on the GPU: a request gives the same bits alone, in a mix of concurrent
requests and under a tight memory budget, equal to the plain fused filter_project call and,
for queries without transcendental operators, to the oracle."""
import numpy as np
import pytest

import helpers as H
import oracle as O
import ralgpu as R
from ralgpu import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served():
    tabs = W.served_tables(6, seed=41, min_rows=1_000, max_rows=300_000)
    qs = W.served_queries(tabs, 16, seed=41)
    host = [W.served_table_host(t) for t in tabs]
    dev = [H.to_device(h) for h in host]
    return tabs, qs, host, dev


def _server(tabs, qs, dev, budget=8 << 30, waves=2):
    srv = R.Server(budget_bytes=budget, max_waves=waves, max_wave_requests=256)
    tids = [srv.add_table(d) for d in dev]
    qids = [srv.add_query(tids[q.table], q.filter, q.project) for q in qs]
    srv.start()
    return srv, qids


def _same_bits(a: R.Column, b: R.Column, what: str):
    assert a.size == b.size, f"{what}: {a.size} rows vs {b.size}"
    assert (a.valid is None) == (b.valid is None), f"{what}: mask presence"
    va, vb = a.valid_bools(), b.valid_bools()
    assert np.array_equal(va, vb), f"{what}: masks differ"
    x, y = a.to_numpy()[va], b.to_numpy()[va]
    assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), f"{what}: data differ"
    assert a.null_count == b.null_count, f"{what}: null_count {a.null_count} vs {b.null_count}"


def _alone(srv, qid):
    rid = srv.submit(qid, keep=True)
    return srv.result(rid, qid)


def _transcendental(q):
    return "SIN(" in q.project or "COS(" in q.project or "SIN(" in q.filter or "COS(" in q.filter


def test_each_query_alone_matches_filter_project_and_oracle(served):
    tabs, qs, host, dev = served
    srv, qids = _server(tabs, qs, dev)
    checked = 0
    for i, (q, qid) in enumerate(zip(qs, qids)):
        got = _alone(srv, qid)
        plain = R.filter_project(dev[q.table], q.filter, q.project)
        assert len(got) == len(plain)
        for k, (g, p) in enumerate(zip(got, plain)):
            _same_bits(g, p, f"query {i} output {k} vs filter_project")
        if _transcendental(q):
            continue
        ef = O.process_filter(H.to_oracle(host[q.table]), q.filter)
        ep = O.execute_project_plan(ef, q.project)
        for k, (g, e) in enumerate(zip(got, ep)):
            H.assert_columns_equal(g, e, what=f"query {i} output {k} vs oracle")
        checked += 1
    assert checked >= 4
    srv.close()


def test_results_are_the_same_alone_and_in_the_mix(served):
    tabs, qs, host, dev = served
    srv, qids = _server(tabs, qs, dev)
    alone = {i: _alone(srv, qids[i]) for i in range(len(qs))}
    rng = np.random.default_rng(3)
    picks = rng.integers(0, len(qs), 400)
    keep = rng.random(400) < 0.15
    rids = [srv.submit(qids[p], keep=bool(k)) for p, k in zip(picks, keep)]   # all in flight together
    for rid, p, k in zip(rids, picks, keep):
        rows, lat = srv.wait(rid)
        assert rows == alone[p][0].size and lat > 0
        if k:
            got = srv.result(rid, qids[p])
            for j, (g, a) in enumerate(zip(got, alone[p])):
                _same_bits(g, a, f"query {p} output {j} in the mix")
        else:
            srv.release(rid)
    st = srv.stats()
    assert st["completed"] >= 400 + len(qs)
    assert st["waves"] < st["completed"]          # requests shared waves
    srv.close()


def test_tight_budget_admits_fewer_requests_and_changes_nothing(served):
    tabs, qs, host, dev = served
    srv0, qids0 = _server(tabs, qs, dev)
    alone = {i: _alone(srv0, qids0[i]) for i in range(len(qs))}
    srv0.close()
    table_bytes = sum(c.size * R.dtypes.WIDTH[c.dtype] + R.valid_alloc_size(c.size) for d in dev for c in d)
    # room for about two of the largest requests at a time
    biggest = max(t.rows for t in tabs) * 64
    budget = table_bytes + 2 * biggest
    srv, qids = _server(tabs, qs, dev, budget=budget, waves=3)
    rids = [(srv.submit(qids[i % len(qs)], keep=True), i % len(qs)) for i in range(3 * len(qs))]
    for rid, i in rids:
        got = srv.result(rid, qids[i])
        for j, (g, a) in enumerate(zip(got, alone[i])):
            _same_bits(g, a, f"query {i} output {j} under the budget")
    st = srv.stats()
    assert st["peak_reserved"] <= budget - table_bytes
    srv.close()


def test_trace_reports_latency_and_rows(served):
    tabs, qs, host, dev = served
    srv, qids = _server(tabs, qs, dev)
    alone_rows = [_alone(srv, q)[0].size for q in qids]
    qi, arr = W.served_trace(300, 2000.0, len(qs), seed=5)
    lat, rows, makespan = srv.run_trace([qids[i] for i in qi], arr)
    assert np.all(lat > 0) and makespan > 0
    assert [int(r) for r in rows] == [alone_rows[i] for i in qi]
    srv.close()


def test_many_large_requests_in_one_wave():
    """Requests of thousands of chunks each, all admitted into the same waves: every chunk's
    look-back finds its predecessor running (no timeouts) and each count equals the alone run."""
    tabs = W.served_tables(2, seed=77, min_rows=3_000_000, max_rows=5_000_000)
    qs = W.served_queries(tabs, 6, seed=77)
    dev = [H.to_device(W.served_table_host(t)) for t in tabs]
    srv, qids = _server(tabs, qs, dev, budget=40 << 30)
    alone = [srv.wait(srv.submit(q))[0] for q in qids]
    rids = [(srv.submit(qids[i % len(qids)]), i % len(qids)) for i in range(96)]
    for rid, i in rids:
        rows, _ = srv.wait(rid, timeout_s=300.0)
        assert rows == alone[i]
        srv.release(rid)
    st = srv.stats()
    assert st["max_wave_requests"] > 8
    srv.close()


def test_requests_sliced_over_many_waves_give_the_same_bits(served, monkeypatch):
    """A wave budget far below one table: every request runs as many slices, each chunk's
    look-back continuing from the status words a previous wave left (no request runs solo)."""
    tabs, qs, host, dev = served
    monkeypatch.setenv("RAL_SERVER_SOLO_ROWS", "0")
    srv0, qids0 = _server(tabs, qs, dev)
    alone = {i: _alone(srv0, qids0[i]) for i in range(len(qs))}
    srv0.close()
    srv = R.Server(budget_bytes=8 << 30, max_waves=3, max_wave_requests=64, wave_rows=5000)
    tids = [srv.add_table(d) for d in dev]
    qids = [srv.add_query(tids[q.table], q.filter, q.project) for q in qs]
    srv.start()
    rids = [(srv.submit(qids[i], keep=True), i) for i in range(len(qs))]
    for rid, i in rids:
        got = srv.result(rid, qids[i])
        for j, (g, a) in enumerate(zip(got, alone[i])):
            _same_bits(g, a, f"query {i} output {j} sliced")
    assert srv.stats()["waves"] > 3 * len(qs)
    srv.close()


def test_empty_and_one_row_tables():
    """A request over an empty table keeps 0 rows; over a one-row table, the row or nothing."""
    import numpy as np
    from ralgpu import dtypes as D
    t0 = [R.Column.from_numpy(np.zeros(0, dtype=np.int32), D.GDF_INT32, np.zeros(0, dtype=bool)),
          R.Column.from_numpy(np.zeros(0), D.GDF_FLOAT64, None)]
    t1 = [R.Column.from_numpy(np.array([7], dtype=np.int32), D.GDF_INT32, np.array([True])),
          R.Column.from_numpy(np.array([2.5]), D.GDF_FLOAT64, None)]
    srv = R.Server(budget_bytes=1 << 30)
    a, b = srv.add_table(t0), srv.add_table(t1)
    fq, pq = "LogicalFilter(condition=[>($0, 5)])", "LogicalProject(x=[*($1, 2)], y=[$0])"
    qa, qb = srv.add_query(a, fq, pq), srv.add_query(b, fq, pq)
    qc = srv.add_query(b, "LogicalFilter(condition=[<($0, 5)])", pq)
    srv.start()
    assert srv.wait(srv.submit(qa))[0] == 0
    got = srv.result(srv.submit(qb, keep=True), qb)
    assert got[0].size == 1 and got[0].to_numpy()[0] == 5.0 and got[1].to_numpy()[0] == 7
    assert srv.wait(srv.submit(qc))[0] == 0
    srv.close()


def test_large_requests_run_solo_with_the_same_bits(served, monkeypatch):
    """Requests over tables of at least RAL_SERVER_SOLO_ROWS rows run alone on the standalone fused
    kernel, the others batched beside them (or alone when nothing else waits): every result equals
    the batched-only server's, and every large request ran solo."""
    tabs, qs, host, dev = served
    monkeypatch.setenv("RAL_SERVER_SOLO_ROWS", "0")
    srv0, qids0 = _server(tabs, qs, dev, waves=3)
    alone = {i: _alone(srv0, qids0[i]) for i in range(len(qs))}
    assert srv0.stats()["solo"] == 0
    srv0.close()
    cut = int(np.median([t.rows for t in tabs]))
    monkeypatch.setenv("RAL_SERVER_SOLO_ROWS", str(cut))
    srv, qids = _server(tabs, qs, dev, waves=3)
    big = [tabs[q.table].rows >= cut for q in qs]
    assert any(big) and not all(big)
    rids = [(srv.submit(qids[i % len(qs)], keep=True), i % len(qs)) for i in range(4 * len(qs))]
    for rid, i in rids:
        got = srv.result(rid, qids[i])
        for j, (g, a) in enumerate(zip(got, alone[i])):
            _same_bits(g, a, f"query {i} output {j} solo={big[i]}")
    st = srv.stats()
    assert st["solo"] >= sum(big[i] for _, i in rids)
    srv.close()


def test_a_request_alone_runs_solo(served):
    """With nothing else waiting a request of any size runs on the standalone kernel, with the
    same bits as ral_filter_project."""
    tabs, qs, host, dev = served
    srv, qids = _server(tabs, qs, dev, waves=2)
    small = min(range(len(qs)), key=lambda i: tabs[qs[i].table].rows)
    s0 = srv.stats()["solo"]
    got = _alone(srv, qids[small])
    assert srv.stats()["solo"] == s0 + 1
    plain = R.filter_project(dev[qs[small].table], qs[small].filter, qs[small].project)
    for k, (g, p) in enumerate(zip(got, plain)):
        _same_bits(g, p, f"output {k}")
    srv.close()


def test_served_transcendentals_match_the_oracle_within_2_ulp():
    """Served item functions with sin / cos / atan / ln in the projection against the oracle's
    process_filter + execute_project_plan, within 2 ulp."""
    from ralgpu import dtypes as D
    rng = np.random.default_rng(72)
    n = 250_000
    host = [(D.GDF_INT32, rng.integers(-100, 100, n).astype(np.int32), rng.random(n) >= 0.05),
            (D.GDF_FLOAT64, rng.uniform(0.01, 3.0, n), rng.random(n) >= 0.05)]
    dev = H.to_device(host)
    fq = "LogicalFilter(condition=[>($0, -20)])"
    projects = ["LogicalProject(s=[SIN($1)], c=[COS($1)], k=[$0])",
                "LogicalProject(a=[ATAN($1)], l=[LN($1)])"]
    srv = R.Server(budget_bytes=4 << 30, max_waves=2, max_wave_requests=64)
    tid = srv.add_table(dev)
    qids = [srv.add_query(tid, fq, pq) for pq in projects]
    srv.start()
    ef = O.process_filter(H.to_oracle(host), fq)
    for qid, pq in zip(qids, projects):
        got = _alone(srv, qid)
        ep = O.execute_project_plan(ef, pq)
        for k, (g, e) in enumerate(zip(got, ep)):
            H.assert_columns_equal(g, e, tol_ulp=H.ULP_TOL, what=f"served {pq} output {k}")
    srv.close()
