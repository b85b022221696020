"""Date and timestamp literals against DATE64 columns: filters and projections through the fused
kernels, compared with the oracle.  The literal is the DATE64 milliseconds that
get_scalar_from_string (src/CalciteExpressionParsing.cpp:337-417) intends: "%Y-%m-%d %H:%M:%S" by
mktime in the local time zone (a bare date at 00:00:00)."""
import time

import numpy as np
import pytest

import oracle as O
import ralgpu as R
from ralgpu import dtypes as D

from helpers import to_device, to_oracle

pytestmark = pytest.mark.gpu


def _frame(n, seed):
    rng = np.random.default_rng(seed)
    lo = int(time.mktime((1990, 1, 1, 0, 0, 0, 0, 0, 0))) * 1000
    hi = int(time.mktime((2030, 1, 1, 0, 0, 0, 0, 0, 0))) * 1000
    ms = rng.integers(lo, hi, n)
    # a share of rows exactly on the literals' instants, where < and <= differ
    on = rng.random(n) < 0.05
    ms[on] = int(time.mktime((2019, 1, 1, 0, 0, 0, 0, 0, 0))) * 1000
    return [(D.GDF_DATE64, ms, rng.random(n) >= 0.05), (D.GDF_INT32, rng.integers(0, 100, n), None),
            (D.GDF_DATE32, rng.integers(0, 20000, n), None)]


FILTERS = [
    "LogicalFilter(condition=[<($0, 2019-01-01 00:00:00)])",
    "LogicalFilter(condition=[<=($0, 2019-01-01)])",
    "LogicalFilter(condition=[AND(>=($0, 1994-01-01), <($0, 1995-01-01 12:30:00), <($1, 50))])",
    "LogicalFilter(condition=[OR(=($0, 2019-01-01 00:00:00), >($0, 2029-06-30 23:59:59))])",
]


@pytest.mark.parametrize("fq", FILTERS)
def test_date_filters(fq):
    spec = _frame(300_001, len(fq))
    got = R.process_filter(to_device(spec), fq)
    exp = O.process_filter(to_oracle(spec), fq)
    assert got[0].size == exp[0].size and exp[0].size > 0
    for g, e in zip(got, exp):
        np.testing.assert_array_equal(g.valid_bools(), e.valid_bools())
        m = e.valid_bools()
        np.testing.assert_array_equal(g.to_numpy()[m], e.data[m])
        assert g.null_count == e.null_count


def test_date_projection_behind_a_filter():
    spec = _frame(200_003, 9)
    fq = "LogicalFilter(condition=[>=($0, 2000-01-01)])"
    pq = "LogicalProject(EXPR$0=[-($0, 2000-01-01 00:00:00)], EXPR$1=[/(-($0, 2000-01-01), 86400000)])"
    got = R.filter_project(to_device(spec), fq, pq)
    f = O.process_filter(to_oracle(spec), fq)
    exp = O.execute_project_plan(f, pq)
    for g, e in zip(got, exp):
        assert g.size == e.size
        np.testing.assert_array_equal(g.valid_bools(), e.valid_bools())
        m = e.valid_bools()
        np.testing.assert_array_equal(g.to_numpy()[m], e.data[m])
