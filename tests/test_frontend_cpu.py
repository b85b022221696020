"""The library's C++ front end emits the same register programs as the oracle's
restatement of the reference emitter (src/LogicalFilter.cpp:44-268)."""
import random

import pytest

import ralgpu
from ralgpu import RalError
from oracle import frontend as fe
from golden import reference_kats as K

BIN = ["=", "<>", ">", ">=", "<", "<=", "+", "-", "*", "/", "POWER", "MOD", "AND", "OR"]
UN = ["NOT", "SIN", "ASIN", "COS", "ACOS", "TAN", "ATAN", "FLOOR", "CEIL", "ABS", "LOG10", "LN",
      "EXTRACT(FLAG(YEAR), ", "EXTRACT(FLAG(MONTH), ", "EXTRACT(FLAG(DAY), "]


def rand_expr(rng, depth, ncols):
    if depth == 0 or rng.random() < 0.25:
        return f"${rng.randrange(ncols)}"
    r = rng.random()
    if r < 0.15:
        u = rng.choice(UN)
        inner = rand_expr(rng, depth - 1, ncols)
        return (u + inner + ")") if u.endswith(", ") else f"{u}({inner})"
    op = rng.choice(BIN)
    if op in ("AND", "OR") and rng.random() < 0.4:
        args = [rand_expr(rng, depth - 1, ncols) for _ in range(rng.randint(3, 5))]
        return f"{op}({', '.join(args)})"
    a = rand_expr(rng, depth - 1, ncols)
    b = rand_expr(rng, depth - 1, ncols)
    k = rng.random()
    if k < 0.2:
        a = rng.choice(["1", "-7", "0.05", "2.5e3", "100"])
    elif k < 0.4:
        b = rng.choice(["3", "-1", "0.5", "1e-3", "24"])
    return f"{op}({a}, {b})"


def oracle_plan(expr, pos, nout, nin, remap):
    plan = fe.Plan()
    fe.add_expression_to_plan(expr, pos, nout, nin, plan, remap)
    return plan


def same(expr, pos=0, nout=1, nin=4, remap=(0, 1, 2, 3)):
    o = oracle_plan(expr, pos, nout, nin, list(remap))
    g = ralgpu.add_expression_to_plan(expr, pos, nout, nin, list(remap))
    assert g["left"] == o.left, expr
    assert g["right"] == o.right, expr
    assert g["outputs"] == o.outputs, expr
    assert g["operators"] == o.operators, expr
    assert g["unary_operators"] == o.unary_operators, expr
    for gs, os_ in zip(g["left_scalars"] + g["right_scalars"], o.left_scalars + o.right_scalars):
        if os_ is fe.JUNK:
            continue
        assert gs.dtype == os_.dtype and gs.value == os_.value and gs.is_valid == os_.is_valid, expr


@pytest.mark.parametrize("expr", [e for e, _ in K.LOGICAL_FILTER_KATS] + [c for c, _, _ in K.WHERE_KATS])
def test_reference_expressions(expr):
    same(expr)


@pytest.mark.parametrize("expr", [
    "AND(OR(AND(>=($2, 24), <($1, 0.05)), =(MOD($0, 7), 3)), <($3, 1200))",
    "+(*($1, -(1, $1)), $2)",
    "CASE(IS NOT NULL($0), $0, -1)",
    "IS NOT NULL($3)",
    "IS NULL($0)",
    "+(CAST($0):DOUBLE, 1.5)",
    "EXTRACT(FLAG(YEAR), $3)",
    "FLOOR(*($1, 10))",
    "OR(=($0, 1), =($0, 2), =($0, 3), =($0, 4), =($0, 5))",
])
def test_handpicked(expr):
    same(expr)


def test_random_trees():
    rng = random.Random(1234)
    checked = 0
    for _ in range(600):
        expr = rand_expr(rng, 4, 6)
        if expr.startswith("$"):
            continue
        same(expr, nin=6, remap=list(range(6)))
        checked += 1
    assert checked > 400


def test_multi_output_positions():
    # a LogicalProject with three evaluated expressions shares registers like the reference
    for k, expr in enumerate(["+($0, $1)", "*(+($0, 1), -($1, 2))", "MOD($2, 7)"]):
        same(expr, pos=k, nout=3, nin=3, remap=[0, 1, 2])


@pytest.mark.parametrize("expr", [
    ">($3, 1995-03-15)",
    "<($3, 2019-01-01 00:00:00)",
    "AND(>=($3, 1994-01-01), <($3, 1995-01-01 12:30:00))",
    "+($3, 2000-02-29)",
])
def test_date_literals(expr):
    """Date and timestamp literals become DATE64 scalars (milliseconds from mktime) in both front
    ends, the time part staying with its date."""
    same(expr)
    g = ralgpu.add_expression_to_plan(expr, 0, 1, 4, [0, 1, 2, 3])
    dates = [s for s in g["right_scalars"] if s.dtype == fe.GDF_DATE64]
    assert dates and all(s.value % 1000 == 0 for s in dates)


def test_date_literal_value():
    import time
    g = ralgpu.add_expression_to_plan("<($3, 2019-01-01 06:30:15)", 0, 1, 4, [0, 1, 2, 3])
    want = int(time.mktime((2019, 1, 1, 6, 30, 15, 0, 0, 0))) * 1000
    assert g["right_scalars"][0].value == want


@pytest.mark.parametrize("expr", ["+(1, 2)", "SIN(2)", "LIKE($0, 'a%')", "=($0, 'abc')", "+($0, null)",
                                  "+($0)", "*($0, $1, $2)", ">($3, 1995-13-40)"])
def test_rejected(expr):
    with pytest.raises((RalError, fe.FrontendError)):
        fe_plan = oracle_plan(expr, 0, 1, 4, [0, 1, 2, 3])  # noqa: F841  (the oracle rejects too)
    with pytest.raises(RalError):
        ralgpu.add_expression_to_plan(expr, 0, 1, 4, [0, 1, 2, 3])


DT = [fe.GDF_INT8, fe.GDF_INT16, fe.GDF_INT32, fe.GDF_INT64, fe.GDF_FLOAT32, fe.GDF_FLOAT64, fe.GDF_DATE32,
      fe.GDF_DATE64]


def test_output_types_random():
    rng = random.Random(99)
    for _ in range(400):
        frame = [rng.choice(DT) for _ in range(6)]
        expr = rand_expr(rng, 3, 6)
        if expr.startswith("$"):
            continue
        try:
            exp = fe.get_output_type_expression(frame, expr)
        except fe.FrontendError:
            with pytest.raises(RalError):
                ralgpu.get_output_type_expression(frame, expr)
            continue
        assert ralgpu.get_output_type_expression(frame, expr) == exp, (frame, expr)


def test_project_output_types():
    frame = [fe.GDF_INT32, fe.GDF_FLOAT64, fe.GDF_INT64]
    q = "LogicalProject(a=[$0], b=[+($0, $1)], c=[>($2, 5)], d=[$2], e=[*($0, 2)])"
    types, evald = ralgpu.project_output_types(frame, q)
    pp = fe.parse_project_plan(frame, q)
    assert evald == [k == "expr" for k, _ in pp.columns]
    exp = []
    for kind, v in pp.columns:
        exp.append(pp.output_types[v] if kind == "expr" else frame[v])
    assert types == exp


def test_is_not_null_in_a_projection_is_rejected_like_the_reference():
    """The reference's projection rewrite drops " NOT NULL" before parsing, so IS NOT NULL outside
    the CASE(IS NOT NULL(x), x, y) pattern is an unknown operator there; both sides reject it."""
    import ralgpu
    from oracle import frontend as fe
    frame = [ralgpu.dtypes.GDF_INT64, ralgpu.dtypes.GDF_FLOAT64]
    q = "LogicalProject(a=[+($0, 1)], b=[IS NOT NULL($1)])"
    with pytest.raises(ralgpu.RalError):
        ralgpu.parse_project_plan(frame, q)
    with pytest.raises(fe.FrontendError):
        fe.parse_project_plan(frame, q)
    ok = "LogicalProject(a=[CASE(IS NOT NULL($1), $1, 0)], b=[IS NULL($1)])"
    assert len(ralgpu.parse_project_plan(frame, ok)["evaluated_dtypes"]) == 2
    assert len(fe.parse_project_plan(frame, ok).output_types) == 2
