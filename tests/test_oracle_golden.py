"""Pins the CPU oracle against the reference's own known-answer tests."""
import numpy as np
import pytest

import oracle as O
from oracle import frontend as fe
from golden import reference_kats as K


def _cols(spec):
    cols = []
    for s in spec:
        if len(s) == 3:
            cols.append(O.make_column(s[1], s[0], s[2]))
        else:
            cols.append(O.make_column(s[1], s[0]))
    return cols


def _fmt6(v):
    return f"{float(v):.6g}"


def _run_program_kat(kat, compat=False):
    ins = [O.make_column(v, t, [True] * len(v)) for t, v in kat["inputs"]]
    n = ins[0].size
    outs = [O.alloc_column(t, n) for t in kat["outputs"]]
    ls = [fe.Scalar(t, v) for t, v in kat["lscalars"]]
    rs = [fe.Scalar(t, v) for t, v in kat["rscalars"]]
    O.perform_operation(outs, ins, kat["left"], kat["right"], kat["outs"], kat["final"], kat["ops"],
                        kat["uops"], ls, rs, float_literal_compat=compat)
    return outs


@pytest.mark.parametrize("kat", K.PROGRAM_KATS, ids=lambda k: k["name"])
def test_program_kats(kat):
    outs = _run_program_kat(kat)
    for col, exp in zip(outs, kat["expected"]):
        got = col.data
        if kat["fmt6"]:
            assert [_fmt6(v) for v in got] == [_fmt6(v) for v in exp]
        else:
            np.testing.assert_array_equal(got, np.asarray(exp).astype(got.dtype))
        assert col.valid_bools().all()


def test_float_literal_compat_reproduces_shipped_conversion():
    """interpreter_ops.cuh:167-168 converts 2.33 to int 2 and the kernel reads those bits as a
    double (~1e-323), so the shipped kernel returns sin(y) instead of sin(y)+2.33."""
    kat = [k for k in K.PROGRAM_KATS if k["name"] == "TEST_02"][0]
    outs = _run_program_kat(kat, compat=True)
    y = np.array([(i + 1) * 10.0 for i in range(10)], dtype=np.float32).astype(np.float64)
    np.testing.assert_allclose(outs[1].data, np.sin(y).astype(np.float32), rtol=1e-6)


@pytest.mark.parametrize("expr,expected", K.LOGICAL_FILTER_KATS, ids=[e for e, _ in K.LOGICAL_FILTER_KATS])
def test_logical_filter_kats(expr, expected):
    frame = [O.make_column(v, t, [True] * len(v)) for t, v in K.LOGICAL_FILTER_FRAME]
    out = O.alloc_column(K.INT8, 32)
    out = O.evaluate_expression(frame, expr, out)
    np.testing.assert_array_equal(out.data, expected.astype(np.int8))


@pytest.mark.parametrize("cond,cols,mask", K.WHERE_KATS, ids=[c for c, _, _ in K.WHERE_KATS])
def test_where_kats(cond, cols, mask):
    frame = [O.make_column(v, t, [True] * len(v)) for t, v in K.WHERE_FRAME]
    res = O.process_filter(frame, f"LogicalFilter(condition=[{cond}])")
    for c in cols:
        np.testing.assert_array_equal(res[c].data, K.WHERE_FRAME[c][1][mask].astype(np.int32))


@pytest.mark.parametrize("cond,expected", K.WHERE_F64_KATS, ids=[c for c, _ in K.WHERE_F64_KATS])
def test_where_f64_kats(cond, expected):
    frame = [O.make_column(K.SWINGS, K.FLOAT64), O.make_column(K.TRACTIONS, K.FLOAT64)]
    res = O.process_filter(frame, f"LogicalFilter(condition=[{cond}])")
    np.testing.assert_array_equal(res[0].data, np.asarray(expected, dtype=np.float64))


@pytest.mark.parametrize("kat", K.IS_NULL_KATS, ids=lambda k: k["name"])
def test_is_null_kats(kat):
    frame = _cols(kat["frame"])
    res = O.process_filter(frame, f"LogicalFilter(condition=[{kat['condition']}])")
    for col, (vals, valids) in zip(res, kat["expected"]):
        vb = col.valid_bools()
        np.testing.assert_array_equal(vb, np.asarray(valids, dtype=bool))
        np.testing.assert_array_equal(col.data[vb], np.asarray(vals, dtype=np.int32)[vb])


@pytest.mark.parametrize("query,expected", K.PROJECT_KATS, ids=["plus", "coalesce"])
def test_project_kats(query, expected):
    frame = _cols(K.EMPS)
    res = O.execute_project_plan(frame, query)
    for col, (vals, valids) in zip(res, expected):
        vb = col.valid_bools()
        np.testing.assert_array_equal(vb, np.asarray(valids, dtype=bool))
        np.testing.assert_array_equal(col.data[vb], np.asarray(vals, dtype=col.data.dtype)[vb])
        assert col.null_count == int((~vb).sum())


@pytest.mark.parametrize("kat", K.AGG_KATS, ids=lambda k: k["name"])
def test_oracle_aggregation_without_group_by(kat):
    """The oracle's process_aggregate against the reference's aggregation known-answer tests."""
    frame = [O.make_column(v, t, m) for t, v, m in K.PARTKEY]
    if kat["filter"]:
        frame = O.process_filter(frame, kat["filter"])
    got = O.process_aggregate(frame, K.AGG_QUERY)
    assert len(got) == len(kat["expected"])
    for g, (t, valid, value) in zip(got, kat["expected"]):
        assert g.dtype == t and g.is_valid == valid
        if valid:
            assert g.value == value


@pytest.mark.parametrize("query,literal", K.CATEGORY_KATS, ids=["exists", "missing"])
def test_oracle_string_category_filter(query, literal):
    """The reference's NVCategory filter tests: rows whose string sorts below the literal; a missing
    literal is added to the dictionary and the codes follow."""
    x = list(range(100, 100 + len(K.CATEGORY_STRINGS)))
    frame = [O.make_column(x, fe.GDF_INT32), O.make_category_column(K.CATEGORY_STRINGS)]
    out = O.process_filter(frame, query)
    assert out[0].data.tolist() == [v for v, s in zip(x, K.CATEGORY_STRINGS) if s < literal]
    assert O.decode_category(out[1]) == [s for s in K.CATEGORY_STRINGS if s < literal]
    assert (literal.encode() in frame[1].category)
