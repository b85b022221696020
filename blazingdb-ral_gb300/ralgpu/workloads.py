"""Synthetic workloads of the expression path, with the shapes and value
distributions the benchmark configurations name.  The reference ships no
dataset for this path, so every input is seeded synthetic data.

  plain_vm     1M rows:  c0 int64 U[0,1e6), c1 float64 U[0,1) with 10% nulls,
               c2 int32 U[1,50], c3 date32 U[0,2400); filter
               ((c2>=24 AND c1<0.05) OR c0%7=3) AND c3<1200, then project
               c1*(1-c1)+c2
  fused_project 200M rows: a,b int64 U[-2^40,2^40), x float64 N(0,1),
               y float64 U[1,100), k int32 U[0,1000), 5% nulls each; a 12-op
               program (add, mul, div, mod, compare, CASE-style select, abs,
               floor) with outputs f1, f2 (float64) and i1 (int64)
  filter_gather 500M rows: int32 U[0,10000), int64, float32, float64, date32,
               bool8; predicate <($0, T) with T = 100 / 5000 / 9900 for
               selectivity 1% / 50% / 99%; every column gathered
  batched      256 programs of 4-48 operators (uniform over arithmetic /
               compare / logical / unary), each over its own table of
               log-uniform [1e3, 5e7] rows and 2-8 int32/int64/float32/float64
               columns with 0-20% nulls
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import dtypes as D

SEED = 20261203

# ---- plain_vm -------------------------------------------------------------------------------

PLAIN_VM_FILTER = ("LogicalFilter(condition=[AND(OR(AND(>=($2, 24), <($1, 0.05)), =(MOD($0, 7), 3)), "
                   "<($3, 1200))])")
PLAIN_VM_PROJECT = "LogicalProject(EXPR$0=[+(*($1, -(1, $1)), $2)])"
PLAIN_VM_DTYPES = [D.GDF_INT64, D.GDF_FLOAT64, D.GDF_INT32, D.GDF_DATE32]


def plain_vm_host(n: int, seed: int = SEED):
    """[(dtype, values, valid_bools or None)] for the plain_vm frame."""
    rng = np.random.default_rng(seed)
    c0 = rng.integers(0, 1_000_000, n, dtype=np.int64)
    c1 = rng.random(n)
    v1 = rng.random(n) >= 0.10
    c2 = rng.integers(1, 51, n).astype(np.int32)
    c3 = rng.integers(0, 2400, n).astype(np.int32)
    return [(D.GDF_INT64, c0, None), (D.GDF_FLOAT64, c1, v1), (D.GDF_INT32, c2, None), (D.GDF_DATE32, c3, None)]


# ---- fused_project --------------------------------------------------------------------------

@dataclass
class ProgramSpec:
    input_dtypes: List[int]
    output_dtypes: List[int]
    left: List[int]
    right: List[int]
    outputs: List[int]
    final: List[int]
    ops: List[int]
    uops: List[int]
    lscalars: list = field(default_factory=list)
    rscalars: list = field(default_factory=list)


def fused_project_program() -> ProgramSpec:
    """Registers: $0=a $1=b $2=x $3=y $4=k; outputs f1=5, f2=6, i1=7; temporaries from 8."""
    I64 = (D.GDF_INT64, 0)
    J = (D.GDF_INT32, 0)
    L, R, O, B, U, RS = [], [], [], [], [], []

    def bin_(l, r, o, op, rs=J):
        L.append(l); R.append(r); O.append(o); B.append(op); U.append(D.BLZ_INVALID_UNARY); RS.append(rs)

    def un(l, o, op):
        L.append(l); R.append(-1); O.append(o); B.append(D.GDF_INVALID_BINARY); U.append(op); RS.append(J)

    bin_(2, 3, 8, D.GDF_MUL)                 # t1 = x * y
    bin_(2, 3, 9, D.GDF_DIV)                 # t2 = x / y
    bin_(8, 9, 5, D.GDF_ADD)                 # f1 = t1 + t2
    bin_(1, -2, 8, D.GDF_GREATER, I64)       # c  = b > 0
    un(2, 9, D.BLZ_FLOOR)                    # t3 = floor(x)
    bin_(3, 2, 10, D.GDF_SUB)                # t4 = y - x
    un(10, 10, D.BLZ_ABS)                    # t5 = |t4|
    bin_(9, 10, 9, D.GDF_SUB)                # t6 = t3 - t5
    bin_(8, 9, 8, D.GDF_MUL)                 # t7 = c * t6
    bin_(10, 8, 6, D.GDF_ADD)                # f2 = t5 + t7   (c ? floor(x) : |y-x|, arithmetic form)
    bin_(4, -2, 9, D.GDF_ADD, (D.GDF_INT64, 1))  # t8 = k + 1
    bin_(0, 9, 7, D.GDF_MOD)                 # i1 = a % t8
    return ProgramSpec(
        input_dtypes=[D.GDF_INT64, D.GDF_INT64, D.GDF_FLOAT64, D.GDF_FLOAT64, D.GDF_INT32],
        output_dtypes=[D.GDF_FLOAT64, D.GDF_FLOAT64, D.GDF_INT64],
        left=L, right=R, outputs=O, final=[5, 6, 7], ops=B, uops=U,
        lscalars=[J] * len(L), rscalars=RS)


# The same projection as RexNode text over the same five columns ($0=a $1=b $2=x $3=y $4=k), behind
# a LogicalFilter on k: the fused filter + project at 200M rows.
FILTER_PROJECT_PROJECT = ("LogicalProject(f1=[+(*($2, $3), /($2, $3))], "
                          "f2=[+(ABS(-($3, $2)), *(>($1, 0), -(FLOOR($2), ABS(-($3, $2)))))], "
                          "i1=[MOD($0, +($4, 1))])")


def filter_project_filter(selectivity: float) -> str:
    """k is uniform in [0, 1000): <($4, 1000 s) keeps a fraction s of the rows."""
    return f"LogicalFilter(condition=[<($4, {int(round(1000 * selectivity))})])"


def fused_project_host(n: int, seed: int = SEED, null_rate: float = 0.05):
    rng = np.random.default_rng(seed)
    lim = 1 << 40
    a = rng.integers(-lim, lim, n, dtype=np.int64)
    b = rng.integers(-lim, lim, n, dtype=np.int64)
    x = rng.standard_normal(n)
    y = rng.uniform(1.0, 100.0, n)
    k = rng.integers(0, 1000, n).astype(np.int32)
    vals = [a, b, x, y, k]
    dts = fused_project_program().input_dtypes
    return [(t, v, rng.random(n) >= null_rate) for t, v in zip(dts, vals)]


def fused_project_device(n: int, seed: int = SEED, null_rate: float = 0.05, device="cuda"):
    """Same distributions generated on the GPU (no host copy of 200M-row columns).
    Returns [(dtype, data tensor, packed valid tensor, null_count)]."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    lim = 1 << 40
    out = []
    a = torch.randint(-lim, lim, (n,), generator=g, device=device, dtype=torch.int64)
    b = torch.randint(-lim, lim, (n,), generator=g, device=device, dtype=torch.int64)
    x = torch.randn(n, generator=g, device=device, dtype=torch.float64)
    y = torch.rand(n, generator=g, device=device, dtype=torch.float64) * 99.0 + 1.0
    k = torch.randint(0, 1000, (n,), generator=g, device=device, dtype=torch.int32)
    for t, v in zip(fused_project_program().input_dtypes, [a, b, x, y, k]):
        valid, nulls = random_valid_mask(n, null_rate, g, device)
        out.append((t, v, valid, nulls))
    return out


def random_valid_mask(n: int, null_rate: float, g, device="cuda"):
    """Packed LSB-first mask (padded to 64 bytes) with independent Bernoulli nulls, built on the GPU."""
    import torch
    from .column import valid_alloc_size
    bits = (torch.rand(n, generator=g, device=device) >= null_rate)
    nulls = int(n - int(bits.sum().item()))
    pad = (-n) % 8
    if pad:
        bits = torch.cat([bits, torch.zeros(pad, dtype=torch.bool, device=device)])
    w = torch.tensor([1, 2, 4, 8, 16, 32, 64, 128], dtype=torch.uint8, device=device)
    packed = (bits.view(-1, 8).to(torch.uint8) * w).sum(dim=1, dtype=torch.uint8)
    buf = torch.zeros(valid_alloc_size(n), dtype=torch.uint8, device=device)
    buf[:packed.numel()] = packed
    return buf, nulls


# ---- filter_gather --------------------------------------------------------------------------

FILTER_GATHER_DTYPES = [D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64, D.GDF_DATE32, D.GDF_BOOL8]
FILTER_THRESHOLDS = {0.01: 100, 0.50: 5000, 0.99: 9900}


def filter_gather_query(selectivity: float) -> str:
    return f"LogicalFilter(condition=[<($0, {FILTER_THRESHOLDS[selectivity]})])"


def filter_gather_host(n: int, seed: int = SEED, null_rate: Optional[float] = None):
    rng = np.random.default_rng(seed)
    c0 = rng.integers(0, 10000, n).astype(np.int32)
    c1 = rng.integers(-(1 << 62), 1 << 62, n, dtype=np.int64)
    c2 = rng.standard_normal(n).astype(np.float32)
    c3 = rng.standard_normal(n)
    c4 = rng.integers(0, 20000, n).astype(np.int32)
    c5 = (rng.random(n) < 0.5).astype(np.int8)
    vals = [c0, c1, c2, c3, c4, c5]
    out = []
    for t, v in zip(FILTER_GATHER_DTYPES, vals):
        m = None if null_rate is None else (rng.random(n) >= null_rate)
        out.append((t, v, m))
    return out


def filter_gather_device(n: int, seed: int = SEED, device="cuda", null_rate: Optional[float] = None):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    c0 = torch.randint(0, 10000, (n,), generator=g, device=device, dtype=torch.int32)
    c1 = torch.randint(-(1 << 62), 1 << 62, (n,), generator=g, device=device, dtype=torch.int64)
    c2 = torch.randn(n, generator=g, device=device, dtype=torch.float32)
    c3 = torch.randn(n, generator=g, device=device, dtype=torch.float64)
    c4 = torch.randint(0, 20000, (n,), generator=g, device=device, dtype=torch.int32)
    c5 = (torch.rand(n, generator=g, device=device) < 0.5).to(torch.int8)
    out = []
    for t, v in zip(FILTER_GATHER_DTYPES, [c0, c1, c2, c3, c4, c5]):
        if null_rate is None:
            out.append((t, v, None, 0))
        else:
            valid, nulls = random_valid_mask(n, null_rate, g, device)
            out.append((t, v, valid, nulls))
    return out


# ---- batched: many independent programs over uneven tables ---------------------------------

BATCH_DTYPES = [D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64]
BATCH_ARITH = ["+", "-", "*", "/", "MOD"]
BATCH_COMPARE = ["=", "<>", "<", ">", "<=", ">="]
BATCH_LOGICAL = ["AND", "OR", "NOT"]
# IS NOT NULL is left out: inside a LogicalProject the reference's expression-list rewrite
# turns it into an unknown operator (only CASE(IS NOT NULL(x), x, y) survives, as COALESCE)
BATCH_UNARY = ["FLOOR", "CEIL", "ABS", "SIN", "COS", "IS NULL"]


@dataclass
class BatchTable:
    """One program of the batched mix: its table shape and its LogicalProject text."""
    rows: int
    dtypes: List[int]
    null_rates: List[float]
    project: str
    n_ops: int
    seed: int


def random_rex(rng, k: int, n_cols: int, literal_ok: bool = True) -> str:
    """A RexNode call tree with exactly k operators; the category of each operator is uniform
    over arithmetic / compare / logical / unary.  Every operator has a column below it: the
    emitter takes no unary operator on a literal and no binary operator on two literals."""
    if k == 0:
        if literal_ok and rng.random() < 0.2:
            return str(int(rng.integers(1, 100))) if rng.random() < 0.5 else f"{rng.integers(1, 400) / 4.0:.2f}"
        return f"${int(rng.integers(0, n_cols))}"
    cat = int(rng.integers(0, 4))
    if cat == 3 or (cat == 2 and rng.random() < 1 / 3):
        op = "NOT" if cat == 2 else BATCH_UNARY[int(rng.integers(0, len(BATCH_UNARY)))]
        if op.startswith("IS ") and k > 1:
            # the VM tests the mask of an input column, not of an intermediate register
            op = BATCH_UNARY[int(rng.integers(0, len(BATCH_UNARY) - 1))]
        return f"{op}({random_rex(rng, k - 1, n_cols, False)})"
    ops = BATCH_ARITH if cat == 0 else BATCH_COMPARE if cat == 1 else ["AND", "OR"]
    op = ops[int(rng.integers(0, len(ops)))]
    kl = int(rng.integers(0, k))
    left = random_rex(rng, kl, n_cols)
    right = random_rex(rng, k - 1 - kl, n_cols, not (kl == 0 and not left.startswith("$")))
    return f"{op}({left}, {right})"


def batched_mix(n_programs: int = 256, seed: int = SEED, min_rows: float = 1e3, max_rows: float = 5e7,
                min_ops: int = 4, max_ops: int = 48) -> List[BatchTable]:
    """The batched workload: each program runs over its own table with a log-uniform row count,
    2-8 columns drawn from int32/int64/float32/float64 with 0-20% nulls, and 4-48 operators
    split over 1-3 projected expressions."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n_programs):
        rows = int(round(math.exp(rng.uniform(math.log(min_rows), math.log(max_rows)))))
        nc = int(rng.integers(2, 9))
        dts = [BATCH_DTYPES[int(i)] for i in rng.integers(0, len(BATCH_DTYPES), nc)]
        nr = [float(rng.uniform(0.0, 0.2)) for _ in range(nc)]
        n_ops = int(rng.integers(min_ops, max_ops + 1))
        n_expr = int(rng.integers(1, min(3, n_ops) + 1))
        cuts = sorted(rng.choice(np.arange(1, n_ops), n_expr - 1, replace=False).tolist()) if n_expr > 1 else []
        parts = np.diff([0] + cuts + [n_ops]).tolist()
        exprs = [random_rex(rng, int(k), nc) for k in parts]
        project = "LogicalProject(" + ", ".join(f"e{i}=[{e}]" for i, e in enumerate(exprs)) + ")"
        out.append(BatchTable(rows, dts, nr, project, n_ops, int(rng.integers(0, 2**31))))
    return out


def _batch_values_np(rng, dtype: int, n: int) -> np.ndarray:
    if dtype == D.GDF_INT32:
        return rng.integers(-1000, 1000, n, dtype=np.int32)
    if dtype == D.GDF_INT64:
        return rng.integers(-(1 << 20), 1 << 20, n, dtype=np.int64)
    if dtype == D.GDF_FLOAT32:
        return rng.uniform(-100, 100, n).astype(np.float32)
    return rng.normal(0.0, 100.0, n)


def batched_table_host(t: BatchTable, rows: Optional[int] = None):
    """Host columns of one table: list of (dtype, values, valid bools or None)."""
    rng = np.random.default_rng(t.seed)
    n = t.rows if rows is None else rows
    cols = []
    for dt, nr in zip(t.dtypes, t.null_rates):
        v = _batch_values_np(rng, dt, n)
        valid = rng.random(n) >= nr if nr > 0 else None
        cols.append((dt, v, valid))
    return cols


def batched_table_device(t: BatchTable, device="cuda"):
    """Device columns of one table: list of (dtype, tensor, packed mask or None, null count)."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(t.seed)
    n = t.rows
    cols = []
    for dt, nr in zip(t.dtypes, t.null_rates):
        if dt == D.GDF_INT32:
            v = torch.randint(-1000, 1000, (n,), generator=g, device=device, dtype=torch.int32)
        elif dt == D.GDF_INT64:
            v = torch.randint(-(1 << 20), 1 << 20, (n,), generator=g, device=device, dtype=torch.int64)
        elif dt == D.GDF_FLOAT32:
            v = torch.rand(n, generator=g, device=device, dtype=torch.float32) * 200 - 100
        else:
            v = torch.randn(n, generator=g, device=device, dtype=torch.float64) * 100
        if nr > 0:
            valid, nulls = random_valid_mask(n, nr, g, device)
        else:
            valid, nulls = None, 0
        cols.append((dt, v, valid, nulls))
    return cols


# ---- served: prepared filter + project queries over resident tables -------------------------

SERVED_DTYPES = [D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64, D.GDF_DATE32]
SERVED_NULL_RATE = 0.05


@dataclass
class ServedTable:
    rows: int
    dtypes: List[int]
    seed: int


@dataclass
class ServedQuery:
    table: int
    filter: str
    project: str
    n_ops: int


def served_tables(n_tables: int = 24, seed: int = SEED, min_rows: float = 1e4, max_rows: float = 1e8) -> List[ServedTable]:
    """Resident tables: log-uniform row counts, 4-8 columns of int32/int64/float32/float64/date32."""
    rng = np.random.default_rng(seed + 1)
    out = []
    for _ in range(n_tables):
        rows = int(round(math.exp(rng.uniform(math.log(min_rows), math.log(max_rows)))))
        nc = int(rng.integers(4, 9))
        dts = [SERVED_DTYPES[int(i)] for i in rng.integers(0, len(SERVED_DTYPES), nc)]
        out.append(ServedTable(rows, dts, int(rng.integers(0, 2**31))))
    return out


def _served_literal(rng, dtype: int) -> str:
    """A literal inside the column's value range, so that comparisons keep a fraction of rows."""
    if dtype == D.GDF_INT32:
        return str(int(rng.integers(-900, 900)))
    if dtype == D.GDF_INT64:
        return str(int(rng.integers(-(1 << 19), 1 << 19)))
    if dtype == D.GDF_DATE32:
        return str(int(rng.integers(1000, 19000)))
    if dtype == D.GDF_FLOAT32:
        return f"{rng.uniform(-90, 90):.2f}"
    return f"{rng.normal(0, 60):.2f}"


def random_predicate(rng, k: int, dtypes: List[int]) -> str:
    """A condition with exactly k operators whose root is a comparison or AND / OR."""
    if k == 1:
        c = int(rng.integers(0, len(dtypes)))
        op = BATCH_COMPARE[int(rng.integers(2, 6))]
        return f"{op}(${c}, {_served_literal(rng, dtypes[c])})"
    if k >= 3 and rng.random() < 0.5:
        a = int(rng.integers(1, k - 1))
        op = "AND" if rng.random() < 0.6 else "OR"
        return f"{op}({random_predicate(rng, a, dtypes)}, {random_predicate(rng, k - 1 - a, dtypes)})"
    op = BATCH_COMPARE[int(rng.integers(2, 6))]
    return f"{op}({random_rex(rng, k - 1, len(dtypes), False)}, {int(rng.integers(-50, 50))})"


def served_queries(tables: List[ServedTable], n_queries: int = 96, seed: int = SEED, min_ops: int = 4,
                   max_ops: int = 32) -> List[ServedQuery]:
    """Prepared queries: a LogicalFilter and a LogicalProject over one table, 4-32 operators in
    all (1 or more in the condition, the rest over 1-3 projected expressions), plus at times a
    column passed through."""
    rng = np.random.default_rng(seed + 2)
    out = []
    for _ in range(n_queries):
        ti = int(rng.integers(0, len(tables)))
        dts = tables[ti].dtypes
        n_ops = int(rng.integers(min_ops, max_ops + 1))
        kf = int(rng.integers(1, min(8, n_ops - 1) + 1))
        kp = n_ops - kf
        n_expr = int(rng.integers(1, min(3, kp) + 1))
        cuts = sorted(rng.choice(np.arange(1, kp), n_expr - 1, replace=False).tolist()) if n_expr > 1 else []
        parts = np.diff([0] + cuts + [kp]).tolist()
        exprs = [f"e{i}=[{random_rex(rng, int(k), len(dts))}]" for i, k in enumerate(parts)]
        if rng.random() < 0.5:
            exprs.append(f"c{len(exprs)}=[${int(rng.integers(0, len(dts)))}]")
        out.append(ServedQuery(ti, f"LogicalFilter(condition=[{random_predicate(rng, kf, dts)}])",
                               "LogicalProject(" + ", ".join(exprs) + ")", n_ops))
    return out


def served_trace(n_requests: int, rate: float, n_queries: int, seed: int = SEED):
    """Poisson arrivals at `rate` requests/s; each request runs a query drawn uniformly."""
    rng = np.random.default_rng(seed + 3)
    gaps = rng.exponential(1.0 / rate, n_requests)
    arrivals = np.cumsum(gaps) - gaps[0]
    queries = rng.integers(0, n_queries, n_requests).astype(np.int32)
    return queries, arrivals


def served_table_host(t: ServedTable, rows: Optional[int] = None):
    """Host columns of a served table: list of (dtype, values, valid bools)."""
    rng = np.random.default_rng(t.seed)
    n = t.rows if rows is None else rows
    cols = []
    for dt in t.dtypes:
        if dt == D.GDF_DATE32:
            v = rng.integers(0, 20000, n, dtype=np.int32)
        else:
            v = _batch_values_np(rng, dt, n)
        cols.append((dt, v, rng.random(n) >= SERVED_NULL_RATE))
    return cols


def served_table_device(t: ServedTable, device="cuda"):
    """Device columns of a served table: list of (dtype, tensor, packed mask, null count)."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(t.seed)
    n = t.rows
    cols = []
    for dt in t.dtypes:
        if dt == D.GDF_INT32:
            v = torch.randint(-1000, 1000, (n,), generator=g, device=device, dtype=torch.int32)
        elif dt == D.GDF_DATE32:
            v = torch.randint(0, 20000, (n,), generator=g, device=device, dtype=torch.int32)
        elif dt == D.GDF_INT64:
            v = torch.randint(-(1 << 20), 1 << 20, (n,), generator=g, device=device, dtype=torch.int64)
        elif dt == D.GDF_FLOAT32:
            v = torch.rand(n, generator=g, device=device, dtype=torch.float32) * 200 - 100
        else:
            v = torch.randn(n, generator=g, device=device, dtype=torch.float64) * 100
        valid, nulls = random_valid_mask(n, SERVED_NULL_RATE, g, device)
        cols.append((dt, v, valid, nulls))
    return cols


# ---- delimited text (scan -> filter) ----------------------------------------------------------
# A lineitem-like '|'-delimited table in fixed-width fields, so that a large one is built with
# vectorised digit arithmetic: orderkey INT64 (10 digits), partkey INT32 (7), quantity INT32 (2),
# extendedprice FLOAT64 (8.2), discount FLOAT64 (0.dd), tax FLOAT32 (0.dd), shipdate DATE64
# (YYYY-MM-DD between 1992 and 1998), commitdate DATE32.
TEXT_DTYPES = [D.GDF_INT64, D.GDF_INT32, D.GDF_INT32, D.GDF_FLOAT64, D.GDF_FLOAT64, D.GDF_FLOAT32, D.GDF_DATE64,
               D.GDF_DATE32]
# TPC-H Q6's conditions over the scan of quantity, extendedprice, discount and shipdate
TEXT_PROJECTIONS = [2, 3, 4, 6]
TEXT_FILTER = ("LogicalFilter(condition=[AND(>=($3, 1994-01-01), <($3, 1995-01-01), >=($2, 0.05), <=($2, 0.07), "
               "<($0, 24))])")


def _digits(v: np.ndarray, width: int) -> np.ndarray:
    """(n, width) ASCII digits of non-negative integers, zero-padded."""
    out = np.empty((v.shape[0], width), dtype=np.uint8)
    x = v.astype(np.int64).copy()
    for k in range(width - 1, -1, -1):
        out[:, k] = (x % 10).astype(np.uint8) + 48
        x //= 10
    return out


def _date_chars(days: np.ndarray) -> np.ndarray:
    """(n, 10) YYYY-MM-DD of days since 1970-01-01."""
    d = np.datetime64("1970-01-01") + days.astype("timedelta64[D]")
    y = d.astype("datetime64[Y]").astype(np.int64) + 1970
    m = (d.astype("datetime64[M]").astype(np.int64) % 12) + 1
    dd = (d - d.astype("datetime64[M]")).astype(np.int64) + 1
    dash = np.full((days.shape[0], 1), ord("-"), dtype=np.uint8)
    return np.concatenate([_digits(y, 4), dash, _digits(m, 2), dash, _digits(dd, 2)], axis=1)


TEXT_ROW_BYTES = 66


def _lineitem_draws(n: int, seed: int):
    rng = np.random.default_rng(seed)
    price = rng.integers(90000, 10500000, n)              # cents
    disc = rng.integers(0, 11, n)                         # hundredths
    tax = rng.integers(0, 9, n)
    ship = rng.integers(8036, 10591, n)                   # 1992-01-02 .. 1998-12-31
    okey, pkey, qty = rng.integers(1, 6_000_000_000, n), rng.integers(1, 2_000_000, n), rng.integers(1, 51, n)
    commit = ship + rng.integers(-60, 60, n)
    return okey, pkey, qty, price, disc, tax, ship, commit


def lineitem_values(n: int, seed: int = SEED):
    """The column values of the lineitem-like table (TEXT_DTYPES), as text_table spells them."""
    okey, pkey, qty, price, disc, tax, ship, commit = _lineitem_draws(n, seed)
    # the nearest double of d.dd is price / 100 rounded once (the division of two exact values)
    return [okey.astype(np.int64), pkey.astype(np.int32), qty.astype(np.int32), price / 100.0, disc / 100.0,
            (tax / 100.0).astype(np.float32), ship.astype(np.int64) * 86_400_000, commit.astype(np.int32)]


LINEITEM_NAMES = ["orderkey", "partkey", "quantity", "extendedprice", "discount", "tax", "shipdate", "commitdate"]


def lineitem_parquet(n: int, seed: int = SEED) -> bytes:
    """The lineitem-like table as a Parquet file (required columns, 1Mi-row row groups)."""
    vals = lineitem_values(n, seed)
    return parquet_bytes([(nm, dt, v, None) for nm, dt, v in zip(LINEITEM_NAMES, TEXT_DTYPES, vals)])


def text_table(n: int, seed: int = SEED, values: bool = False):
    """n rows of the lineitem-like table, each ended by '\\n' (fixed width: 66 bytes a row); with
    values=True also the column values the text spells (for a check that needs no parse)."""
    bar = np.full((n, 1), ord("|"), dtype=np.uint8)
    point = np.full((n, 1), ord("."), dtype=np.uint8)
    zero = np.full((n, 1), ord("0"), dtype=np.uint8)
    okey, pkey, qty, price, disc, tax, ship, commit = _lineitem_draws(n, seed)
    parts = [_digits(okey, 10), bar, _digits(pkey, 7), bar,
             _digits(qty, 2), bar, _digits(price // 100, 8), point, _digits(price % 100, 2), bar,
             zero, point, _digits(disc, 2), bar, zero, point, _digits(tax, 2), bar, _date_chars(ship), bar,
             _date_chars(commit), np.full((n, 1), 10, dtype=np.uint8)]
    text = np.concatenate(parts, axis=1).tobytes()
    if not values:
        return text
    return text, lineitem_values(n, seed)


def text_table_varied(n: int, seed: int = SEED) -> bytes:
    """A small table of the same schema that exercises the field rules: signs, spaces, empty and
    unreadable fields, exponents, short rows, blank lines and '\\r\\n' line ends; a header line."""
    import random
    rng = random.Random(seed)
    out = ["orderkey|partkey|quantity|extendedprice|discount|tax|shipdate|commitdate"]
    for r in range(n):
        if rng.random() < 0.03:
            out.append("")
            continue
        def pick(f, bad):
            x = rng.random()
            return "" if x < 0.04 else (bad if x < 0.06 else f)
        y, m, d = rng.randint(1992, 1998), rng.randint(1, 12), rng.randint(1, 28)
        fields = [pick(str(rng.randint(-(1 << 40), 1 << 40)), "12x"),
                  pick(f" {rng.randint(-99999, 99999)} ", "+"),
                  pick(str(rng.randint(1, 50)), "1.5"),
                  pick(rng.choice([f"{rng.randint(0, 10**7)}.{rng.randint(0, 99):02d}", f"{rng.randint(1, 999)}e{rng.randint(-5, 5)}",
                                   f"-{rng.random():.6f}", f"{rng.randint(0, 10**12)}"]), "1.2.3"),
                  pick(f"0.{rng.randint(0, 10):02d}", "x"),
                  pick(f"{rng.randint(0, 8) / 100:.2f}", "."),
                  pick(f"{y:04d}-{m:02d}-{d:02d}" + (f" {rng.randint(0, 23):02d}:{rng.randint(0, 59):02d}:00"
                                                     if rng.random() < 0.2 else ""), "1995-02-30"),
                  pick(f"{y:04d}-{m:02d}-{d:02d}", "19950101")]
        if rng.random() < 0.05:
            fields = fields[:rng.randint(1, 7)]
        out.append("|".join(fields) + ("\r" if rng.random() < 0.1 else ""))
    return ("\n".join(out) + ("\n" if rng.random() < 0.5 else "")).encode()


# ---- Parquet files (scan -> filter over Parquet pages) ---------------------------------------
# A minimal writer of the Apache Parquet format (flat schema, data pages v1 of PLAIN values or
# dictionary indices, definition levels of optional columns in the RLE / bit-packed hybrid,
# uncompressed or literal-only Snappy), for the tests and the benchmark, which run where no Parquet
# library is installed.  Metadata is Thrift's compact protocol.

_PQ_TYPE = {D.GDF_INT32: 1, D.GDF_DATE32: 1, D.GDF_INT64: 2, D.GDF_DATE64: 2, D.GDF_FLOAT32: 4, D.GDF_FLOAT64: 5}
_PQ_CONVERTED = {D.GDF_DATE32: 6, D.GDF_DATE64: 9}   # DATE, TIMESTAMP_MILLIS


class _Compact:
    def __init__(self):
        self.b = bytearray()
        self.last = [0]

    def varint(self, v: int):
        while True:
            x = v & 0x7F
            v >>= 7
            if v:
                self.b.append(x | 0x80)
            else:
                self.b.append(x)
                return

    @staticmethod
    def zigzag(v: int) -> int:
        return (v << 1) ^ (v >> 63) if v < 0 else v << 1

    def field(self, fid: int, ftype: int):
        delta = fid - self.last[-1]
        if 0 < delta <= 15:
            self.b.append((delta << 4) | ftype)
        else:
            self.b.append(ftype)
            self.varint(self.zigzag(fid))
        self.last[-1] = fid

    def i32(self, fid, v):
        self.field(fid, 5)
        self.varint(self.zigzag(v))

    def i64(self, fid, v):
        self.field(fid, 6)
        self.varint(self.zigzag(v))

    def binary(self, fid, bs: bytes):
        self.field(fid, 8)
        self.varint(len(bs))
        self.b += bs

    def begin(self, fid):
        self.field(fid, 12)
        self.last.append(0)

    def end(self):
        self.b.append(0)
        self.last.pop()

    def list_header(self, fid, etype, n):
        self.field(fid, 9)
        if n < 15:
            self.b.append((n << 4) | etype)
        else:
            self.b.append(0xF0 | etype)
            self.varint(n)

    def elem_begin(self):
        self.last.append(0)

    def elem_end(self):
        self.b.append(0)
        self.last.pop()


def _def_levels(valid: np.ndarray) -> bytes:
    """Definition levels (bit width 1) in the RLE / bit-packed hybrid: runs of 16 or more equal
    levels as RLE runs, the rest bit-packed in groups of 8."""
    out = bytearray()
    n = valid.shape[0]
    i = 0
    enc = _Compact()
    while i < n:
        j = i
        while j < n and valid[j] == valid[i]:
            j += 1
        if j - i >= 16:
            enc.b = bytearray()
            enc.varint((j - i) << 1)
            out += enc.b + bytes([1 if valid[i] else 0])
            i = j
            continue
        # bit-packed: up to the next long run (whole groups of 8; the last group padded)
        k = i
        while k < n:
            r = k
            while r < n and valid[r] == valid[k]:
                r += 1
            if r - k >= 16 and (k - i) % 8 == 0 and k > i:
                break
            k = r if r - k < 16 else k + 8
            if k > n:
                k = n
        k = min(k, n)
        groups = (k - i + 7) // 8
        bits = np.zeros(groups * 8, dtype=np.uint8)
        bits[:k - i] = valid[i:k]
        enc.b = bytearray()
        enc.varint((groups << 1) | 1)
        out += enc.b + np.packbits(bits, bitorder="little").tobytes()
        i = k
    return len(out).to_bytes(4, "little") + bytes(out)


def _snappy_literals(raw: bytes, length=None) -> bytes:
    """A raw Snappy stream holding `raw` as literal elements only (valid Snappy, no back-references);
    `length` overrides the stream's stated uncompressed length (a malformed stream for tests)."""
    enc = _Compact()
    enc.varint(len(raw) if length is None else length)
    out = bytearray(enc.b)
    for i in range(0, len(raw), 1 << 16):
        n = len(raw[i:i + (1 << 16)]) - 1
        if n < 60:
            out.append(n << 2)
        else:
            out.append(61 << 2)                   # the length - 1 in the next two bytes
            out += n.to_bytes(2, "little")
        out += raw[i:i + (1 << 16)]
    return bytes(out)


def _bit_packed(idx: np.ndarray, bw: int) -> bytes:
    """idx (non-negative, below 2^bw) as one bit-packed run of the RLE / bit-packed hybrid."""
    k = idx.shape[0]
    groups = (k + 7) // 8
    enc = _Compact()
    enc.varint((groups << 1) | 1)
    if bw == 0 or k == 0:
        return bytes(enc.b)
    padded = np.zeros(groups * 8, dtype=np.uint64)
    padded[:k] = idx
    bits = ((padded[:, None] >> np.arange(bw, dtype=np.uint64)) & np.uint64(1)).astype(np.uint8)
    return bytes(enc.b) + np.packbits(bits.reshape(-1), bitorder="little").tobytes()


def _page_header(kind: int, raw_len: int, stored_len: int, rows: int, encoding: int) -> bytes:
    h = _Compact()
    h.i32(1, kind)                        # 0 DATA_PAGE, 2 DICTIONARY_PAGE
    h.i32(2, raw_len)
    h.i32(3, stored_len)
    if kind == 2:
        h.begin(7)                        # DictionaryPageHeader
        h.i32(1, rows)
        h.i32(2, encoding)
    else:
        h.begin(5)                        # DataPageHeader
        h.i32(1, rows)
        h.i32(2, encoding)
        h.i32(3, 3)                       # RLE definition levels
        h.i32(4, 3)
    h.end()
    h.b.append(0)
    return bytes(h.b)


def parquet_bytes(columns, row_group_rows: int = 1 << 20, page_rows: int = 1 << 17, snappy: bool = False,
                  snappy_length_delta: int = 0, dictionary: bool = False, dictionary_max: int = 65536,
                  chunk_bytes: Optional[list] = None) -> bytes:
    """columns: [(name, gdf dtype, values, valid bools or None for a required column)].  snappy=True
    writes SNAPPY chunks whose page bodies are literal-only Snappy streams (snappy_length_delta != 0
    states a wrong uncompressed length in every stream: a malformed file for tests).
    dictionary=True writes a column chunk with at most dictionary_max distinct values (by bit pattern)
    as a PLAIN dictionary page and RLE_DICTIONARY data pages (the indices as one bit-packed run).
    chunk_bytes, when given, receives (column index, bytes) of every column chunk written."""
    n = len(columns[0][2])
    out = bytearray(b"PAR1")
    row_groups = []

    def put(body: bytearray, kind: int, rows: int, encoding: int) -> int:
        raw_len = len(body)
        if snappy:
            body = bytearray(_snappy_literals(bytes(body), raw_len + snappy_length_delta))
        hb = _page_header(kind, raw_len, len(body), rows, encoding)
        out.extend(hb)
        out.extend(body)
        return len(hb) + len(body)

    for r0 in range(0, max(n, 1), row_group_rows):
        r1 = min(n, r0 + row_group_rows)
        chunks = []
        for name, dt, vals, valid in columns:
            start = len(out)
            nbytes = 0
            bits_of = np.dtype(D.NP[dt]).itemsize * 8
            cv = np.ascontiguousarray(np.asarray(vals[r0:r1]).astype(D.NP[dt]))
            cm = None if valid is None else np.asarray(valid[r0:r1], dtype=bool)
            dict_vals = None
            if dictionary and r1 > r0:
                key = cv.view(np.uint32 if bits_of == 32 else np.uint64)
                present = key if cm is None else key[cm]
                uniq, inv = np.unique(present, return_inverse=True)
                if 0 < len(uniq) <= dictionary_max:
                    dict_vals = uniq.view(cv.dtype)
                    bw = int(len(uniq) - 1).bit_length()
                    nbytes += put(bytearray(np.ascontiguousarray(dict_vals).tobytes()), 2, len(uniq), 0)
                    inv_all = np.zeros(r1 - r0, dtype=np.int64)
                    if cm is None:
                        inv_all[:] = inv
                    else:
                        inv_all[cm] = inv
            data_start = len(out)
            for p0 in range(r0, max(r1, r0 + 1), page_rows):
                p1 = min(r1, p0 + page_rows)
                v = cv[p0 - r0:p1 - r0]
                body = bytearray()
                keep = None
                if cm is not None:
                    keep = cm[p0 - r0:p1 - r0]
                    body += _def_levels(keep)
                if dict_vals is not None:
                    ix = inv_all[p0 - r0:p1 - r0]
                    if keep is not None:
                        ix = ix[keep]
                    body += bytes([bw]) + _bit_packed(ix.astype(np.uint64), bw)
                    nbytes += put(body, 0, p1 - p0, 8)
                else:
                    if keep is not None:
                        v = v[keep]
                    body += v.tobytes()
                    nbytes += put(body, 0, p1 - p0, 0)
                if r1 == r0:
                    break
            chunks.append((name, dt, start, nbytes, r1 - r0, data_start if dict_vals is not None else -1))
            if chunk_bytes is not None:
                chunk_bytes.append((len(chunks) - 1, nbytes))
        row_groups.append((r1 - r0, chunks))
        if n == 0:
            break
    m = _Compact()
    m.i32(1, 1)
    m.list_header(2, 12, len(columns) + 1)
    m.elem_begin(); m.binary(4, b"schema"); m.i32(5, len(columns)); m.elem_end()
    for name, dt, vals, valid in columns:
        m.elem_begin()
        m.i32(1, _PQ_TYPE[dt])
        m.i32(3, 0 if valid is None else 1)
        m.binary(4, name.encode())
        if dt in _PQ_CONVERTED:
            m.i32(6, _PQ_CONVERTED[dt])
        m.elem_end()
    m.i64(3, n)
    m.list_header(4, 12, len(row_groups))
    for rows, chunks in row_groups:
        m.elem_begin()
        m.list_header(1, 12, len(chunks))
        total = 0
        for name, dt, start, nbytes, crow, data_start in chunks:
            total += nbytes
            m.elem_begin()
            m.i64(2, start)
            m.begin(3)
            m.i32(1, _PQ_TYPE[dt])
            if data_start >= 0:
                m.list_header(2, 5, 3); m.varint(m.zigzag(0)); m.varint(m.zigzag(3)); m.varint(m.zigzag(8))
            else:
                m.list_header(2, 5, 2); m.varint(m.zigzag(0)); m.varint(m.zigzag(3))
            m.list_header(3, 8, 1); m.varint(len(name)); m.b += name.encode()
            m.i32(4, 1 if snappy else 0)          # codec
            m.i64(5, crow)
            m.i64(6, nbytes)
            m.i64(7, nbytes)
            m.i64(9, data_start if data_start >= 0 else start)
            if data_start >= 0:
                m.i64(11, start)                  # dictionary_page_offset
            m.end()
            m.elem_end()
        m.i64(2, total)
        m.i64(3, rows)
        m.elem_end()
    m.binary(6, b"ralgpu parquet writer")
    m.b.append(0)
    out += m.b + len(m.b).to_bytes(4, "little") + b"PAR1"
    return bytes(out)
