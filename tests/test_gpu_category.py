"""String-category predicates (src/LogicalFilter.cpp:150-211): string literals compared with a
GDF_STRING_CATEGORY column and two category columns compared with each other, through the fused
filter and projection kernels, against the oracle's restatement and the reference's NVCategory
known-answer tests.  Rows are compared as decoded strings and as codes; after a call that adds a
missing literal, the column's rewritten codes and its new dictionary are compared too."""
import numpy as np
import pytest

import oracle as O
import ralgpu as R
from ralgpu import dtypes as D

from golden import reference_kats as K

pytestmark = pytest.mark.gpu


def _pair(strings, x, valids=None):
    col, cat = R.category_column(strings, valids)
    dev = [R.Column.from_numpy(np.asarray(x), D.GDF_INT32), col]
    ora = [O.make_column(x, D.GDF_INT32), O.make_category_column(strings, valids)]
    return dev, ora


@pytest.mark.parametrize("query,literal", K.CATEGORY_KATS, ids=["exists", "missing"])
def test_reference_category_kats(query, literal):
    x = list(range(100, 100 + len(K.CATEGORY_STRINGS)))
    dev, ora = _pair(K.CATEGORY_STRINGS, x)
    out = R.process_filter(dev, query)
    assert out[0].to_numpy().tolist() == [v for v, s in zip(x, K.CATEGORY_STRINGS) if s < literal]
    assert R.decode_category(out[1]) == [s for s in K.CATEGORY_STRINGS if s < literal]
    keys = R.Category(dev[1].category).keys()
    assert literal in keys and keys == sorted(keys)


def _random_strings(rng, n, length, alphabet="abcdefghijklmnopqrstuvwxyz"):
    a = np.array(list(alphabet))
    return ["".join(rng.choice(a, length)) for _ in range(n)]


@pytest.mark.parametrize("cond", ["<($1, 'm')", "=($1, 'q')", ">=($1, 'zz')", "<>($1, 'c')",
                                  "AND(>($1, 'b'), <($1, 'x'), >($0, 5))", "OR(=($1, 'aa'), =($1, 'k'))"])
def test_string_literal_filters(cond):
    rng = np.random.default_rng(len(cond))
    n = 50_000
    strings = _random_strings(rng, n, 1)
    x = rng.integers(0, 10, n)
    valids = rng.random(n) >= 0.05
    dev, ora = _pair(strings, x, valids)
    q = f"LogicalFilter(condition=[{cond}])"
    got = R.process_filter(dev, q)
    exp = O.process_filter(ora, q)
    assert got[0].size == exp[0].size
    np.testing.assert_array_equal(got[0].to_numpy(), exp[0].data)
    assert R.decode_category(got[1]) == O.decode_category(exp[1])
    # the frame column after the call: same dictionary and codes as the oracle's
    assert R.Category(dev[1].category).keys() == [k.decode() for k in ora[1].category]
    np.testing.assert_array_equal(dev[1].to_numpy(), ora[1].data)


def test_two_category_columns_compared():
    rng = np.random.default_rng(5)
    n = 20_000
    a = _random_strings(rng, n, 2, "abcd")
    b = _random_strings(rng, n, 2, "bcde")
    ca, _ = R.category_column(a)
    cb, _ = R.category_column(b)
    oa, ob = O.make_category_column(a), O.make_category_column(b)
    q = "LogicalFilter(condition=[=($0, $1)])"
    got = R.process_filter([ca, cb], q)
    exp = O.process_filter([oa, ob], q)
    assert got[0].size == exp[0].size == sum(1 for s, t in zip(a, b) if s == t)
    assert R.decode_category(got[0]) == O.decode_category(exp[0]) == R.decode_category(got[1])
    # both frame columns now share one merged dictionary
    assert R.Category(ca.category).keys() == R.Category(cb.category).keys() == sorted(set(a) | set(b))


def test_category_filter_project():
    rng = np.random.default_rng(8)
    n = 30_000
    strings = _random_strings(rng, n, 1)
    x = rng.integers(0, 1000, n)
    dev, ora = _pair(strings, x)
    fq = "LogicalFilter(condition=[AND(>=($1, 'f'), <($1, 'p'))])"
    pq = "LogicalProject(x=[$0], y=[$1], z=[*($0, 2)])"
    got = R.filter_project(dev, fq, pq)
    f = O.process_filter(ora, fq)
    exp = O.execute_project_plan(f, pq)
    np.testing.assert_array_equal(got[0].to_numpy(), exp[0].data)
    assert R.decode_category(got[1]) == O.decode_category(exp[1])
    np.testing.assert_array_equal(got[2].to_numpy(), exp[2].data)
