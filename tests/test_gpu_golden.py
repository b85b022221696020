"""The reference's known-answer tests, run through the C ABI on the GPU."""
import numpy as np
import pytest

import ralgpu as R
from golden import reference_kats as K

pytestmark = pytest.mark.gpu


def _fmt6(v):
    return f"{float(v):.6g}"


@pytest.mark.parametrize("kat", K.PROGRAM_KATS, ids=lambda k: k["name"])
def test_program_kats(kat):
    ins = [R.Column.from_numpy(v, t, [True] * len(v)) for t, v in kat["inputs"]]
    n = ins[0].size
    outs = [R.Column.empty(t, n) for t in kat["outputs"]]
    R.perform_operation(outs, ins, kat["left"], kat["right"], kat["outs"], kat["final"], kat["ops"], kat["uops"],
                        [R.Scalar(t, v) for t, v in kat["lscalars"]], [R.Scalar(t, v) for t, v in kat["rscalars"]])
    for col, exp in zip(outs, kat["expected"]):
        got = col.to_numpy()
        if kat["fmt6"]:
            assert [_fmt6(v) for v in got] == [_fmt6(v) for v in exp]
        elif got.dtype.kind == "f" and kat["name"] == "TEST_01_Unary_Operators":
            np.testing.assert_allclose(got, np.asarray(exp, dtype=got.dtype), rtol=2e-7)
        else:
            np.testing.assert_array_equal(got, np.asarray(exp).astype(got.dtype))
        assert col.valid_bools().all()


@pytest.mark.parametrize("expr,expected", K.LOGICAL_FILTER_KATS, ids=[e for e, _ in K.LOGICAL_FILTER_KATS])
def test_logical_filter_kats(expr, expected):
    frame = [R.Column.from_numpy(v, t, [True] * len(v)) for t, v in K.LOGICAL_FILTER_FRAME]
    out = R.Column.empty(K.INT8, 32)
    R.evaluate_expression(frame, expr, out)
    np.testing.assert_array_equal(out.to_numpy(), expected.astype(np.int8))


@pytest.mark.parametrize("cond,cols,mask", K.WHERE_KATS, ids=[c for c, _, _ in K.WHERE_KATS])
def test_where_kats(cond, cols, mask):
    frame = [R.Column.from_numpy(v, t, [True] * len(v)) for t, v in K.WHERE_FRAME]
    res = R.process_filter(frame, f"LogicalFilter(condition=[{cond}])")
    for c in cols:
        np.testing.assert_array_equal(res[c].to_numpy(), K.WHERE_FRAME[c][1][mask].astype(np.int32))


@pytest.mark.parametrize("cond,expected", K.WHERE_F64_KATS, ids=[c for c, _ in K.WHERE_F64_KATS])
def test_where_f64_kats(cond, expected):
    frame = [R.Column.from_numpy(K.SWINGS, K.FLOAT64), R.Column.from_numpy(K.TRACTIONS, K.FLOAT64)]
    res = R.process_filter(frame, f"LogicalFilter(condition=[{cond}])")
    assert res[0].size == len(expected)
    np.testing.assert_array_equal(res[0].to_numpy(), np.asarray(expected, dtype=np.float64))


@pytest.mark.parametrize("kat", K.IS_NULL_KATS, ids=lambda k: k["name"])
def test_is_null_kats(kat):
    frame = [R.Column.from_numpy(v, t, m) for t, v, m in kat["frame"]]
    res = R.process_filter(frame, f"LogicalFilter(condition=[{kat['condition']}])")
    for col, (vals, valids) in zip(res, kat["expected"]):
        vb = col.valid_bools()
        np.testing.assert_array_equal(vb, np.asarray(valids, dtype=bool))
        np.testing.assert_array_equal(col.to_numpy()[vb], np.asarray(vals, dtype=np.int32)[vb])
        assert col.null_count == int((~vb).sum())


@pytest.mark.parametrize("query,expected", K.PROJECT_KATS, ids=["plus", "coalesce"])
def test_project_kats(query, expected):
    frame = [R.Column.from_numpy(v, t, m) for t, v, m in K.EMPS]
    res = R.execute_project_plan(frame, query)
    for col, (vals, valids) in zip(res, expected):
        vb = col.valid_bools()
        np.testing.assert_array_equal(vb, np.asarray(valids, dtype=bool))
        np.testing.assert_array_equal(col.to_numpy()[vb], np.asarray(vals, dtype=np.int32)[vb])
        assert col.null_count == int((~vb).sum())
