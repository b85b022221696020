"""The benchmark's full-size parity checker, exercised on CPU tensors.

bench.parity_check compares a workload's device outputs with the oracle in row chunks (so that a
200M / 500M-row run fits in host memory).  Here the "device" columns are CPU tensors and the
outputs come from the oracle run over the WHOLE input at once: the chunked check must report zero
mismatches, including across chunk boundaries (the kept rows of a chunk land at a running output
offset that is not a multiple of 8), and one planted bit flip in data, validity or the kept count
must be found.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
import ralgpu as R
from ralgpu import workloads as W

import bench


def _dev(oc):
    data = torch.from_numpy(np.ascontiguousarray(oc.data).copy())
    valid = None if oc.valid is None else torch.from_numpy(oc.valid.copy())
    return R.Column(data, valid, oc.dtype, size=oc.size, null_count=oc.null_count)


class _Nout:
    def __init__(self, v):
        self.value = v


def _structs(cols):
    out = []
    for c in cols:
        s = R.column.GdfColumn()
        s.null_count = c.null_count
        out.append(s)
    return out


@pytest.fixture
def small_chunks(monkeypatch):
    monkeypatch.setattr(bench, "PARITY_CHUNK", 4096)


def _filter_ctx(n, sel, project):
    spec = W.fused_project_host(n, seed=5)
    frame = [O.make_column(v, t, m) for t, v, m in spec]
    fq = W.filter_project_filter(sel)
    pq = W.FILTER_PROJECT_PROJECT if project else None
    f = O.process_filter(frame, fq, nthreads=2)
    outs = O.execute_project_plan(f, pq, nthreads=2) if project else f
    for c in outs:
        O.update_null_count(c)
    dev_outs = [_dev(c) for c in outs]
    return {"cols": [_dev(c) for c in frame], "outs": dev_outs, "nout": _Nout(outs[0].size),
            "out_structs": _structs(dev_outs), "fq": fq, "pq": pq}


@pytest.mark.parametrize("project", [False, True])
def test_chunked_filter_parity_is_clean(small_chunks, project):
    ctx = _filter_ctx(3 * 4096 + 999, 0.37, project)
    res = bench.parity_check("filter_project", ctx, 0.37)
    assert res["chunks"] == 4
    assert res["mismatches"] == 0, res
    assert res["rows_out"] == ctx["nout"].value


def test_chunked_filter_parity_finds_planted_errors(small_chunks):
    ctx = _filter_ctx(3 * 4096 + 999, 0.5, True)
    k = ctx["nout"].value
    # a data bit of a valid row in the third chunk's output range
    vb = ctx["outs"][2].valid_bools()
    row = int(np.nonzero(vb[k // 2:])[0][0]) + k // 2
    ctx["outs"][2].data[row] ^= 1
    assert bench.parity_check("filter_project", ctx, 0.5)["detail"]["data"] == 1
    ctx["outs"][2].data[row] ^= 1
    # a validity bit at an odd output offset
    ctx["outs"][0].valid[(k // 3) // 8] ^= np.uint8(1 << ((k // 3) % 8))
    assert bench.parity_check("filter_project", ctx, 0.5)["detail"]["valid"] == 1
    ctx["outs"][0].valid[(k // 3) // 8] ^= np.uint8(1 << ((k // 3) % 8))
    ctx["nout"].value += 1
    assert bench.parity_check("filter_project", ctx, 0.5)["detail"]["rows_out"] == 1


def test_chunked_projection_parity(small_chunks):
    n = 2 * 4096 + 77
    spec = W.fused_project_program()
    host = W.fused_project_host(n, seed=11)
    frame = [O.make_column(v, t, m) for t, v, m in host]
    from oracle import frontend as fe
    outs = [O.alloc_column(t, n) for t in spec.output_dtypes]
    O.perform_operation(outs, frame, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops,
                        [fe.Scalar(*x) for x in spec.lscalars], [fe.Scalar(*x) for x in spec.rscalars])
    ctx = {"cols": [_dev(c) for c in frame], "outs": [_dev(c) for c in outs], "spec": spec}
    res = bench.parity_check("fused_project", ctx, 0.5)
    assert res["mismatches"] == 0, res
    ctx["outs"][1].data[n - 1] = -ctx["outs"][1].data[n - 1] if outs[1].valid_bools()[n - 1] else 0.0
    exp = 1 if outs[1].valid_bools()[n - 1] else 0
    assert bench.parity_check("fused_project", ctx, 0.5)["detail"]["data"] == exp


def test_reference_arm_prints_the_same_config():
    """Both arms describe a workload with the same `config` dict."""
    a = bench.workload_config("filter_gather", 500_000_000, 0.5, 1)
    b = bench.workload_config("filter_gather", 500_000_000, 0.5, 1)
    assert a == b and a["parallelism"] == "replicas x1"
    assert bench.workload_config("fused_project", 200_000_000, 0.5)["rows"] == 200_000_000


def test_chunked_gather_parity(small_chunks):
    rng = np.random.default_rng(2)
    n = 3 * 4096 + 5
    frame = [O.make_column(v, t, m) for t, v, m in W.filter_gather_host(n, seed=3, null_rate=0.1)]
    idx = rng.permutation(n).astype(np.int32)
    outs = [O.materialize_column(c, idx) for c in frame]
    dev_outs = [_dev(c) for c in outs]
    ctx = {"cols": [_dev(c) for c in frame], "outs": dev_outs, "out_structs": _structs(dev_outs),
           "idx": R.Column(torch.from_numpy(idx), None, 3, size=n)}
    res = bench.gather_parity(ctx)
    assert res["mismatches"] == 0, res
    ctx["outs"][3].data[n - 2] += 1.0
    exp = int(outs[3].valid_bools()[n - 2]) if outs[3].valid is not None else 1
    assert bench.gather_parity(ctx)["detail"]["data"] == exp


def test_parquet_cpu_baseline_reads_a_bounded_sample():
    """The Parquet blocks' CPU baseline: the oracle's reader and filter over the first row groups."""
    import bench as B
    from ralgpu import workloads as W
    n = 300_000
    values = W.lineitem_values(n, W.SEED)
    for dictionary in (False, True):
        blob = W.parquet_bytes([(nm, dt, v, None) for nm, dt, v in zip(W.LINEITEM_NAMES, W.TEXT_DTYPES, values)],
                               row_group_rows=100_000, dictionary=dictionary)
        out = B.cpu_parquet(dict(blob=blob, rows=n, row_group_rows=100_000, row_groups=3), budget_s=0.5)
        assert out["kind"] == "port" and out["value"] > 0 and out["cores"] >= 1
        assert "row groups" in out["sample"]


def test_batched_floor_from_the_committed_table():
    """The mix's floor from profiles/batch_mix_fp64.json: FP64-bound, about 87 ms at 2070 MHz."""
    import json
    import os
    import bench as B
    table = json.load(open(os.path.join(B.ROOT, "profiles", "batch_mix_fp64.json")))
    f = B.batch_floor(table, 2070.0, 6782.4)
    assert 80.0 < f["fp64_ms"] < 95.0 and f["hbm_ms"] < f["fp64_ms"]
    assert f["floor_ms"] == max(f["fp64_ms"], f["hbm_ms"])
