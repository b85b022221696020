"""ral_process_aggregate: LogicalAggregate without GROUP BY, expression inputs fused with the
reduction, against the oracle's restatement of the reference flow (evaluate each expression into a
column, then cudf-style reductions) and against the reference's own known-answer tests.

Comparison: dtypes and validity exactly; integer SUM / COUNT and every MIN / MAX exactly (a min or
max is one of the values); a float SUM within the error bound of any summation order,
(n - 1) * 2^-53 * sum(|x|), of the exactly rounded sum; AVG likewise divided by the count.  Two
calls must give identical bits (the device reduction order is fixed).
"""
import numpy as np
import pytest

import oracle as O
import ralgpu as R
from ralgpu import dtypes as D

from golden import reference_kats as K
from helpers import to_device, to_oracle

pytestmark = pytest.mark.gpu

U = 2.0 ** -53


def _check(got, exp, n):
    assert len(got) == len(exp)
    for i, (g, e) in enumerate(zip(got, exp)):
        assert g.dtype == e.dtype, (i, g, e)
        assert bool(g.is_valid) == bool(e.is_valid), (i, g, e)
        if not e.is_valid:
            continue
        if isinstance(e.value, float) and e.float_sum_bound:
            cnt = 1.0 if g.dtype != D.GDF_FLOAT64 or e.float_sum_bound == 0 else None
            tol = max(n - 1, 1) * U * e.float_sum_bound
            assert abs(g.value - e.value) <= tol + 1e-300, (i, g.value, e.value, tol)
        elif isinstance(e.value, float):
            assert g.value == e.value or (np.isnan(g.value) and np.isnan(e.value)), (i, g.value, e.value)
        else:
            assert int(g.value) == int(e.value), (i, g.value, e.value)


def _frame(rng, n, null_rate=0.05):
    lim = 1 << 40
    spec = [
        (D.GDF_INT64, rng.integers(-lim, lim, n), rng.random(n) >= null_rate),
        (D.GDF_INT64, rng.integers(-lim, lim, n), rng.random(n) >= null_rate),
        (D.GDF_FLOAT64, rng.standard_normal(n), rng.random(n) >= null_rate),
        (D.GDF_FLOAT64, rng.uniform(1, 100, n), rng.random(n) >= null_rate),
        (D.GDF_INT32, rng.integers(0, 1000, n), rng.random(n) >= null_rate),
        (D.GDF_FLOAT32, rng.standard_normal(n).astype(np.float32), None),
        (D.GDF_INT8, rng.integers(-100, 100, n), rng.random(n) >= 0.3),
        (D.GDF_INT16, rng.integers(-30000, 30000, n), None),
    ]
    return spec


QUERIES = [
    # the 12-op projection's outputs as aggregate inputs, with bare columns beside them
    "LogicalAggregate(group=[{}], EXPR$0=[SUM(+(*($2, $3), /($2, $3)))], "
    "EXPR$1=[AVG(+(ABS(-($3, $2)), *(>($1, 0), -(FLOOR($2), ABS(-($3, $2))))))], "
    "EXPR$2=[MIN(MOD($0, +($4, 1)))], EXPR$3=[MAX(MOD($0, +($4, 1)))], EXPR$4=[COUNT()], "
    "EXPR$5=[SUM($4)], EXPR$6=[MAX($3)])",
    # every operator on a bare column of every width, with and without nulls
    "LogicalAggregate(group=[{}], a=[SUM($6)], b=[MIN($6)], c=[MAX($6)], d=[AVG($6)], e=[COUNT($6)], "
    "f=[SUM($7)], g=[MIN($7)], h=[MAX($5)], i=[SUM($5)], j=[AVG($0)], k=[MIN($2)])",
    # integer expressions that wrap, comparisons (INT8 results), float32 arithmetic
    "LogicalAggregate(group=[{}], a=[SUM(*($0, $1))], b=[SUM(>($2, 0))], c=[MAX(*($5, 2))], "
    "d=[MIN(-($7, $6))], e=[AVG(+($4, $6))])",
]


@pytest.mark.parametrize("n", [1, 31, 1000, 100_003, 2_000_000])
@pytest.mark.parametrize("q", range(len(QUERIES)))
def test_aggregate_matches_oracle(n, q):
    rng = np.random.default_rng(1000 * q + n)
    spec = _frame(rng, n)
    got = R.process_aggregate(to_device(spec), QUERIES[q])
    exp = O.process_aggregate(to_oracle(spec), QUERIES[q], nthreads=8)
    _check(got, exp, n)
    again = R.process_aggregate(to_device(spec), QUERIES[q])
    for a, b in zip(got, again):
        assert a.is_valid == b.is_valid and (not a.is_valid or a.to_c().data == b.to_c().data)


@pytest.mark.parametrize("kat", K.AGG_KATS, ids=lambda k: k["name"])
def test_aggregate_reference_kats(kat):
    frame = to_device(K.PARTKEY)
    if kat["filter"]:
        frame = R.process_filter(frame, kat["filter"])
    got = R.process_aggregate(frame, K.AGG_QUERY)
    for g, (t, valid, value) in zip(got, kat["expected"]):
        assert g.dtype == t and bool(g.is_valid) == valid
        if valid:
            assert g.value == value


def test_aggregate_all_null_and_empty_inputs():
    n = 5000
    rng = np.random.default_rng(3)
    spec = [(D.GDF_INT32, rng.integers(0, 9, n), np.zeros(n, dtype=bool)),
            (D.GDF_FLOAT64, rng.random(n), None)]
    dev = to_device(spec)
    q = ("LogicalAggregate(group=[{}], a=[SUM($0)], b=[MIN($0)], c=[AVG($0)], d=[COUNT($0)], "
         "e=[SUM(+($0, 1))], f=[COUNT()])")
    got = R.process_aggregate(dev, q)
    exp = O.process_aggregate(to_oracle(spec), q)
    _check(got, exp, n)
    # the bare all-null column's aggregates are null; the evaluated one counts every row
    assert [g.is_valid for g in got] == [False, False, False, True, True, True]
    assert got[3].value == 0 and got[5].value == 0
    empty = [R.Column.empty(D.GDF_INT32, 0, with_valid=False), R.Column.empty(D.GDF_FLOAT64, 0, with_valid=False)]
    got = R.process_aggregate(empty, q)
    assert [g.is_valid for g in got] == [False, False, False, True, False, True]


def test_aggregate_of_200M_row_projection_inputs():
    """The 12-op projection's three outputs summed over 200M device rows, no column written."""
    import torch
    import bench
    from ralgpu import workloads as W
    n = 200_000_000
    cols = [R.Column(d, v, t, n, nn) for t, d, v, nn in W.fused_project_device(n)]
    q = ("LogicalAggregate(group=[{}], f1=[SUM(+(*($2, $3), /($2, $3)))], "
         "i1=[SUM(MOD($0, +($4, 1)))], m=[MIN(MOD($0, +($4, 1)))], c=[COUNT()])")
    got = R.process_aggregate(cols, q)
    torch.cuda.synchronize()
    exp = bench.aggregate_oracle_chunked(cols, q)
    _check(got, exp, n)
