"""Batched execution on the GPU: every program of a batch gives the same bits as its own
perform_operation call, and programs without transcendental operators match the oracle."""
import numpy as np
import pytest

import helpers as H
import oracle as O
import ralgpu as R
from oracle import frontend as fe
from ralgpu import dtypes as D
from ralgpu import workloads as W

pytestmark = pytest.mark.gpu


def _build(mix, rows_cap=None):
    """Per program: plan, host columns, device inputs, batch outputs and plain outputs."""
    out = []
    for t in mix:
        pp = R.parse_project_plan(t.dtypes, t.project)
        host = W.batched_table_host(t, rows=min(t.rows, rows_cap) if rows_cap else None)
        spec = [host[c] for c in pp["input_columns"]]
        dev_in = H.to_device(spec)
        n = dev_in[0].size
        outs_b = [R.Column.empty(dt, n, with_valid=True) for dt in pp["evaluated_dtypes"]]
        outs_p = [R.Column.empty(dt, n, with_valid=True) for dt in pp["evaluated_dtypes"]]
        out.append(dict(t=t, pp=pp, spec=spec, dev_in=dev_in, outs_b=outs_b, outs_p=outs_p, n=n))
    return out


def _args(pp):
    return (pp["left"], pp["right"], pp["outputs"], pp["final_output_positions"], pp["operators"],
            pp["unary_operators"], pp["left_scalars"], pp["right_scalars"])


def _assert_same_bits(a: R.Column, b: R.Column, what: str):
    assert np.array_equal(a.valid_bools(), b.valid_bools()), f"{what}: masks differ"
    m = a.valid_bools()
    x, y = a.to_numpy()[m], b.to_numpy()[m]
    if x.dtype.kind == "f":
        x, y = x.view(np.int64 if x.itemsize == 8 else np.int32), y.view(np.int64 if y.itemsize == 8 else np.int32)
    bad = np.nonzero(x != y)[0]
    assert bad.size == 0, f"{what}: {bad.size} rows differ"


def _has_transcendental(pp):
    return any(u in (D.BLZ_SIN, D.BLZ_COS) for u in pp["unary_operators"])


@pytest.mark.parametrize("seed", [1, 2])
def test_batch_matches_plain_calls_and_oracle(seed):
    import torch
    mix = W.batched_mix(40, seed=seed, min_rows=1, max_rows=200_000)
    progs = _build(mix)
    b = R.Batch()
    for p in progs:
        b.add(p["outs_b"], p["dev_in"], *_args(p["pp"]))
    b.prepare()
    info = b.info()
    assert info["programs"] == len(progs) and info["rows"] == sum(p["n"] for p in progs)
    b.run()
    torch.cuda.synchronize()
    checked = 0
    for q, p in enumerate(progs):
        R.perform_operation(p["outs_p"], p["dev_in"], *_args(p["pp"]))
        for k, (x, y) in enumerate(zip(p["outs_b"], p["outs_p"])):
            _assert_same_bits(x, y, f"program {q} output {k}")
        if _has_transcendental(p["pp"]):
            continue
        ora_in = H.to_oracle(p["spec"])
        ora_out = [O.alloc_column(dt, p["n"]) for dt in p["pp"]["evaluated_dtypes"]]
        pp = p["pp"]
        O.perform_operation(ora_out, ora_in, pp["left"], pp["right"], pp["outputs"], pp["final_output_positions"],
                            pp["operators"], pp["unary_operators"],
                            [fe.Scalar(s.dtype, s.value, s.is_valid) for s in pp["left_scalars"]],
                            [fe.Scalar(s.dtype, s.value, s.is_valid) for s in pp["right_scalars"]], nthreads=8)
        for k, (g, e) in enumerate(zip(p["outs_b"], ora_out)):
            H.assert_columns_equal(g, e, what=f"program {q} output {k} vs oracle", check_null_count=False)
        checked += 1
    assert checked >= 5


def test_batch_graph_replay_and_direct_launch_agree():
    import torch
    mix = W.batched_mix(12, seed=5, min_rows=1000, max_rows=300_000)
    progs = _build(mix)
    b = R.Batch()
    for p in progs:
        b.add(p["outs_b"], p["dev_in"], *_args(p["pp"]))
    b.run(use_graph=True)
    torch.cuda.synchronize()
    first = [[(c.to_numpy().copy(), c.valid_bools().copy()) for c in p["outs_b"]] for p in progs]
    for p in progs:
        for c in p["outs_b"]:
            c.data.fill_(0)
            c.valid.fill_(0)
    for _ in range(3):
        b.run(use_graph=True)
    b.run(use_graph=False)
    torch.cuda.synchronize()
    for q, p in enumerate(progs):
        for k, c in enumerate(p["outs_b"]):
            v, m = first[q][k]
            assert np.array_equal(c.valid_bools(), m)
            assert np.array_equal(c.to_numpy()[m].view(np.uint8), v[m].view(np.uint8)), f"program {q} output {k}"
    info = b.info()
    assert info["registers"] > 0 and info["grid"] > 0


def test_batch_edge_sizes_and_unaligned_views():
    """Tables of 1, 31, 32, 33 and 4097 rows, and inputs that start mid-vector (scalar loads)."""
    import torch
    mix = W.batched_mix(10, seed=9, min_rows=1, max_rows=10)
    rows = [1, 31, 32, 33, 4097, 64, 65, 127, 129, 1000]
    progs = []
    for t, n in zip(mix, rows):
        t.rows = n
    progs = _build(mix)
    # program 0: inputs viewed one element in (misaligned for vector loads)
    p0 = progs[0]
    shifted = []
    for c, (dt, v, m) in zip(p0["dev_in"], p0["spec"]):
        big = R.Column.from_numpy(np.concatenate([v[:1], v]), dt, None if m is None else np.concatenate([m[:1], m]))
        shifted.append(R.Column(big.data[1:], c.valid, dt, c.size, c.null_count))
    p0["dev_in"] = shifted
    b = R.Batch()
    for p in progs:
        b.add(p["outs_b"], p["dev_in"], *_args(p["pp"]))
    b.run()
    torch.cuda.synchronize()
    for q, p in enumerate(progs):
        R.perform_operation(p["outs_p"], p["dev_in"], *_args(p["pp"]))
        for k, (x, y) in enumerate(zip(p["outs_b"], p["outs_p"])):
            _assert_same_bits(x, y, f"program {q} ({p['n']} rows) output {k}")


def test_autotune_records_a_shape_and_batch_still_matches():
    import torch
    mix = W.batched_mix(4, seed=11, min_rows=100_000, max_rows=400_000)
    progs = _build(mix)
    p = progs[0]
    J, U, soft, ms = R.autotune_program(p["outs_b"], p["dev_in"], *_args(p["pp"]))
    assert J in (2, 4, 8, 16) and U in (1, 2) and soft in (False, True) and ms > 0
    b = R.Batch()
    for p in progs:
        b.add(p["outs_b"], p["dev_in"], *_args(p["pp"]))
    b.run()
    torch.cuda.synchronize()
    for q, p in enumerate(progs):
        R.perform_operation(p["outs_p"], p["dev_in"], *_args(p["pp"]))
        for k, (x, y) in enumerate(zip(p["outs_b"], p["outs_p"])):
            _assert_same_bits(x, y, f"program {q} output {k}")


def test_batch_with_empty_tables():
    """Programs over empty tables contribute no work items; the others still run."""
    import torch
    mix = W.batched_mix(6, seed=13, min_rows=100, max_rows=5000)
    mix[1].rows = 0
    mix[4].rows = 0
    progs = _build(mix)
    b = R.Batch()
    for p in progs:
        b.add(p["outs_b"], p["dev_in"], *_args(p["pp"]))
    b.run()
    torch.cuda.synchronize()
    assert b.info()["rows"] == sum(p["n"] for p in progs)
    for q, p in enumerate(progs):
        if p["n"] == 0:
            continue
        R.perform_operation(p["outs_p"], p["dev_in"], *_args(p["pp"]))
        for k, (x, y) in enumerate(zip(p["outs_b"], p["outs_p"])):
            _assert_same_bits(x, y, f"program {q} output {k}")


TRANS = ["SIN", "COS", "TAN", "ATAN", "ASIN", "ACOS", "LN", "LOG10"]


def test_batched_transcendentals_match_the_oracle_within_2_ulp():
    """Batched item functions with sin / cos / tan / atan / asin / acos / ln / log10 against the
    oracle (libm), one transcendental per output so that the per-operation bound applies."""
    import torch
    rng = np.random.default_rng(71)
    progs = []
    for k, op in enumerate(TRANS):
        n = int(rng.integers(1000, 60_000))
        x = rng.uniform(0.01, 0.99, n) if op in ("LN", "LOG10", "ASIN", "ACOS") else rng.uniform(-3, 3, n)
        spec = [(D.GDF_FLOAT64, x, rng.random(n) >= 0.05), (D.GDF_INT32, rng.integers(1, 9, n).astype(np.int32), None)]
        pp = R.parse_project_plan([D.GDF_FLOAT64, D.GDF_INT32],
                                  f"LogicalProject(a=[{op}($0)], b=[{op}($1)])")
        ins = [spec[c] for c in pp["input_columns"]]
        dev_in = H.to_device(ins)
        outs = [R.Column.empty(dt, n, with_valid=True) for dt in pp["evaluated_dtypes"]]
        progs.append(dict(op=op, pp=pp, ins=ins, dev_in=dev_in, outs=outs, n=n))
    b = R.Batch()
    for p in progs:
        b.add(p["outs"], p["dev_in"], *_args(p["pp"]))
    b.prepare()
    b.run()
    torch.cuda.synchronize()
    for p in progs:
        pp = p["pp"]
        ora_out = [O.alloc_column(dt, p["n"]) for dt in pp["evaluated_dtypes"]]
        O.perform_operation(ora_out, H.to_oracle(p["ins"]), pp["left"], pp["right"], pp["outputs"],
                            pp["final_output_positions"], pp["operators"], pp["unary_operators"],
                            [fe.Scalar(s.dtype, s.value, s.is_valid) for s in pp["left_scalars"]],
                            [fe.Scalar(s.dtype, s.value, s.is_valid) for s in pp["right_scalars"]], nthreads=8)
        for k, (g, e) in enumerate(zip(p["outs"], ora_out)):
            H.assert_columns_equal(g, e, tol_ulp=H.ULP_TOL, what=f"batched {p['op']} output {k}",
                                   check_null_count=False)
