"""GPU parity against the CPU oracle, through the C ABI.

Bit-exact for integer, date, comparison and logical results, validity masks,
null counts and compacted row order; bit-exact for + - * / and floor/ceil/abs
on doubles (kernels are built with --fmad=false and explicit _rn intrinsics);
transcendentals within helpers.ULP_TOL ulp.
"""
import numpy as np
import pytest

import oracle as O
import ralgpu as R
from oracle import frontend as fe
from ralgpu import dtypes as D
from ralgpu import workloads as W

import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["fused", "unfused"])
def filter_mode(request, monkeypatch):
    """process_filter / filter_project run as one fused kernel (default) or as the reference's
    three steps (stencil, compaction, gather); both must match the oracle."""
    if request.param == "unfused":
        monkeypatch.setenv("RAL_FILTER_MODE", "unfused")
    else:
        monkeypatch.delenv("RAL_FILTER_MODE", raising=False)
    return request.param


def program_dict(spec: W.ProgramSpec):
    return dict(left=spec.left, right=spec.right, outputs=spec.outputs, final=spec.final, ops=spec.ops,
                uops=spec.uops, lscalars=spec.lscalars, rscalars=spec.rscalars)


# ---- fused_project shape (12 ops, 5 inputs, 3 outputs) ---------------------------------------

@pytest.mark.parametrize("n", [0, 1, 31, 33, 127, 128, 129, 1000, 4097, 100_003])
def test_fused_project_program(n):
    spec = W.fused_project_program()
    inputs = W.fused_project_host(n, seed=11 + n)
    dev, ora = H.run_program_both(inputs, spec.output_dtypes, program_dict(spec))
    for k, (g, e) in enumerate(zip(dev, ora)):
        H.assert_columns_equal(g, e, what=f"output {k}", check_null_count=False)


def test_fused_project_null_counts_async():
    spec = W.fused_project_program()
    n = 50_001
    inputs = W.fused_project_host(n, seed=5)
    dev_in = H.to_device(inputs)
    outs = [R.Column.empty(t, n) for t in spec.output_dtypes]
    nc = R.perform_operation_async(outs, dev_in, spec.left, spec.right, spec.outputs, spec.final, spec.ops,
                                   spec.uops, spec.lscalars, spec.rscalars, want_null_counts=True)
    ora_in = H.to_oracle(inputs)
    ora_out = [O.alloc_column(t, n) for t in spec.output_dtypes]
    O.perform_operation(ora_out, ora_in, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops,
                        [fe.Scalar(*s) for s in spec.lscalars], [fe.Scalar(*s) for s in spec.rscalars])
    for k in range(3):
        assert nc[k] == n - int(ora_out[k].valid_bools().sum())


def test_fused_project_without_masks():
    spec = W.fused_project_program()
    n = 20_000
    inputs = [(t, v, None) for t, v, _ in W.fused_project_host(n, seed=3)]
    dev, ora = H.run_program_both(inputs, spec.output_dtypes, program_dict(spec), out_valid=False)
    for g, e in zip(dev, ora):
        H.assert_columns_equal(g, e, check_null_count=False)


# ---- plain_vm shape: filter then project -----------------------------------------------------

@pytest.mark.parametrize("n", [1, 64, 1000, 1_000_000])
def test_plain_vm_filter_then_project(n, filter_mode):
    spec = W.plain_vm_host(n, seed=21)
    dev = H.to_device(spec)
    ora = H.to_oracle(spec)
    gf = R.process_filter(dev, W.PLAIN_VM_FILTER)
    ef = O.process_filter(ora, W.PLAIN_VM_FILTER)
    for k, (g, e) in enumerate(zip(gf, ef)):
        H.assert_columns_equal(g, e, what=f"filtered column {k}")
    gp = R.execute_project_plan(gf, W.PLAIN_VM_PROJECT)
    ep = O.execute_project_plan(ef, W.PLAIN_VM_PROJECT)
    H.assert_columns_equal(gp[0], ep[0], what="projection")


@pytest.mark.parametrize("n", [1, 1000, 1_000_000])
def test_plain_vm_fused_filter_project(n, filter_mode):
    spec = W.plain_vm_host(n, seed=22)
    dev = H.to_device(spec)
    ora = H.to_oracle(spec)
    got = R.filter_project(dev, W.PLAIN_VM_FILTER, W.PLAIN_VM_PROJECT)
    ef = O.process_filter(ora, W.PLAIN_VM_FILTER)
    ep = O.execute_project_plan(ef, W.PLAIN_VM_PROJECT)
    H.assert_columns_equal(got[0], ep[0], what="fused filter+project")


# ---- filter_gather shape ----------------------------------------------------------------------

@pytest.mark.parametrize("sel", [0.01, 0.50, 0.99])
@pytest.mark.parametrize("null_rate", [None, 0.05])
@pytest.mark.parametrize("n", [777, 1_000_003])
def test_filter_gather(sel, null_rate, n, filter_mode):
    spec = W.filter_gather_host(n, seed=31, null_rate=null_rate)
    dev = H.to_device(spec)
    ora = H.to_oracle(spec)
    q = W.filter_gather_query(sel)
    got = R.process_filter(dev, q)
    exp = O.process_filter(ora, q)
    for k, (g, e) in enumerate(zip(got, exp)):
        H.assert_columns_equal(g, e, what=f"column {k}")


def test_filter_keeps_row_order_and_count(filter_mode):
    n = 300_001
    rng = np.random.default_rng(4)
    keep = rng.random(n) < 0.3
    iota = np.arange(n, dtype=np.int64)
    frame = [R.Column.from_numpy(keep.astype(np.int32), D.GDF_INT32), R.Column.from_numpy(iota, D.GDF_INT64)]
    res = R.process_filter(frame, "LogicalFilter(condition=[=($0, 1)])")
    np.testing.assert_array_equal(res[1].to_numpy(), np.nonzero(keep)[0])


def test_filter_stencil_or_sum_two_and_null_stencil(filter_mode):
    """OR is integer addition: rows matching both sides give 2 (nonzero -> kept); a null stencil drops the row."""
    vals = np.array([1, 2, 3, 4, 5, 6], dtype=np.int32)
    valid = np.array([1, 1, 0, 1, 1, 1], dtype=bool)
    spec = [(D.GDF_INT32, vals, valid), (D.GDF_INT32, vals * 10, None)]
    q = "LogicalFilter(condition=[OR(>($0, 1), <($1, 45))])"
    got = R.process_filter(H.to_device(spec), q)
    exp = O.process_filter(H.to_oracle(spec), q)
    for g, e in zip(got, exp):
        H.assert_columns_equal(g, e)
    assert got[0].size == 5


def test_filter_bare_column_condition(filter_mode):
    stencil = np.array([0, 1, 2, 0, -1, 0, 1], dtype=np.int8)
    sv = np.array([1, 1, 1, 1, 1, 0, 1], dtype=bool)
    spec = [(D.GDF_INT8, stencil, sv), (D.GDF_FLOAT64, np.arange(7) * 1.5, None)]
    q = "LogicalFilter(condition=[$0])"
    got = R.process_filter(H.to_device(spec), q)
    exp = O.process_filter(H.to_oracle(spec), q)
    for g, e in zip(got, exp):
        H.assert_columns_equal(g, e)


def test_filter_empty_frame():
    spec = [(D.GDF_INT32, np.zeros(0, dtype=np.int32), None)]
    got = R.process_filter(H.to_device(spec), "LogicalFilter(condition=[>($0, 1)])")
    assert got[0].size == 0


# ---- null rules ------------------------------------------------------------------------------

def test_null_count_zero_means_all_valid_but_is_null_reads_bits():
    """interpreter_ops.cuh:1314: null_count == 0 -> the validity pass treats the column as all valid;
    IS_NULL (:820-829) still reads the raw bits."""
    n = 200
    rng = np.random.default_rng(9)
    v = rng.random(n) < 0.5
    vals = rng.integers(0, 100, n).astype(np.int32)
    for nc in (0, int((~v).sum())):
        dev = [R.Column.from_numpy(vals, D.GDF_INT32, v, null_count=nc), R.Column.from_numpy(vals, D.GDF_INT32)]
        ora = [O.make_column(vals, D.GDF_INT32, v, null_count=nc), O.make_column(vals, D.GDF_INT32)]
        # out0 = $0 + 1 ; out1 = IS_NULL($0) (op index 1: the :1314 flag lands on column 1)
        prog = dict(left=[0, 0], right=[-2, -1], outputs=[2, 3], final=[2, 3], ops=[D.GDF_ADD, D.GDF_INVALID_BINARY],
                    uops=[D.BLZ_INVALID_UNARY, D.BLZ_IS_NULL], lscalars=[(D.GDF_INT32, 0)] * 2,
                    rscalars=[(D.GDF_INT64, 1), (D.GDF_INT32, 0)])
        go = [R.Column.empty(D.GDF_INT64, n), R.Column.empty(D.GDF_INT8, n)]
        eo = [O.alloc_column(D.GDF_INT64, n), O.alloc_column(D.GDF_INT8, n)]
        R.perform_operation(go, dev, prog["left"], prog["right"], prog["outputs"], prog["final"], prog["ops"],
                            prog["uops"], prog["lscalars"], prog["rscalars"])
        O.perform_operation(eo, ora, prog["left"], prog["right"], prog["outputs"], prog["final"], prog["ops"],
                            prog["uops"], [fe.Scalar(*s) for s in prog["lscalars"]],
                            [fe.Scalar(*s) for s in prog["rscalars"]])
        for g, e in zip(go, eo):
            H.assert_columns_equal(g, e, check_null_count=False)


def test_is_null_in_compound_filter_follows_reference_column_flag(filter_mode):
    """AND(IS NULL($0), >($1, 5)): op 1 is IS_NULL, so the validity pass forces column 1 (not 0) all-valid."""
    n = 64
    rng = np.random.default_rng(2)
    a = rng.integers(0, 10, n).astype(np.int32)
    b = rng.integers(0, 10, n).astype(np.int32)
    va = rng.random(n) < 0.5
    vb = rng.random(n) < 0.7
    spec = [(D.GDF_INT32, a, va), (D.GDF_INT32, b, vb)]
    q = "LogicalFilter(condition=[AND(IS NULL($0), >($1, 5))])"
    got = R.process_filter(H.to_device(spec), q)
    exp = O.process_filter(H.to_oracle(spec), q)
    for g, e in zip(got, exp):
        H.assert_columns_equal(g, e)


def test_coalesce_and_null_scalar():
    n = 1000
    rng = np.random.default_rng(8)
    x = rng.integers(-50, 50, n).astype(np.int64)
    vx = rng.random(n) < 0.6
    y = rng.standard_normal(n)
    spec = [(D.GDF_INT64, x, vx), (D.GDF_FLOAT64, y, None)]
    # out0 = COALESCE($0, $1) ; out1 = $1 * null  (valid 0 everywhere)
    prog = dict(left=[0, 1], right=[1, -3], outputs=[2, 3], final=[2, 3], ops=[D.GDF_COALESCE, D.GDF_MUL],
                uops=[D.BLZ_INVALID_UNARY] * 2, lscalars=[(D.GDF_INT32, 0)] * 2,
                rscalars=[(D.GDF_INT32, 0), (D.GDF_FLOAT64, 0.0, False)])
    dev, ora = H.run_program_both(spec, [D.GDF_INT64, D.GDF_FLOAT64], prog)
    for g, e in zip(dev, ora):
        H.assert_columns_equal(g, e, check_null_count=False)


def test_register_to_column_bit_reinterpretation():
    """write_data reads the slot's bits with the COLUMN's type (interpreter_ops.cuh:317-381)."""
    n = 300
    x = np.linspace(-3, 3, n)
    spec = [(D.GDF_FLOAT64, x, None)]
    prog = dict(left=[0], right=[-2], outputs=[1], final=[1], ops=[D.GDF_ADD], uops=[D.BLZ_INVALID_UNARY],
                lscalars=[(D.GDF_INT32, 0)], rscalars=[(D.GDF_FLOAT64, 0.25)])
    for out_t in (D.GDF_INT32, D.GDF_INT64, D.GDF_INT8):
        dev, ora = H.run_program_both(spec, [out_t], prog)
        H.assert_columns_equal(dev[0], ora[0], check_null_count=False)


# ---- random programs --------------------------------------------------------------------------

IN_TYPES = [D.GDF_INT8, D.GDF_INT16, D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64, D.GDF_DATE32,
            D.GDF_DATE64]
OUT_TYPES = [D.GDF_INT8, D.GDF_INT16, D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64]
EXACT_BIN = [D.GDF_ADD, D.GDF_SUB, D.GDF_MUL, D.GDF_DIV, D.GDF_MOD, D.GDF_EQUAL, D.GDF_NOT_EQUAL, D.GDF_LESS,
             D.GDF_GREATER, D.GDF_LESS_EQUAL, D.GDF_GREATER_EQUAL, D.GDF_COALESCE, D.GDF_FLOOR_DIV]
EXACT_UN = [D.BLZ_FLOOR, D.BLZ_CEIL, D.BLZ_ABS, D.BLZ_NOT, D.BLZ_YEAR, D.BLZ_MONTH, D.BLZ_DAY, D.BLZ_HOUR,
            D.BLZ_MINUTE, D.BLZ_SECOND, D.BLZ_IS_NULL, D.BLZ_IS_NOT_NULL, D.BLZ_INVALID_UNARY]
TRANS_UN = [D.BLZ_SIN, D.BLZ_COS, D.BLZ_TAN, D.BLZ_ATAN, D.BLZ_LN, D.BLZ_LOG, D.BLZ_ASIN, D.BLZ_ACOS, D.BLZ_COTAN]


def rand_values(rng, t, n):
    if t == D.GDF_INT8:
        return rng.integers(-128, 128, n)
    if t == D.GDF_INT16:
        return rng.integers(-30000, 30000, n)
    if t == D.GDF_INT32:
        return rng.integers(-1_000_000, 1_000_000, n)
    if t == D.GDF_INT64:
        v = rng.integers(-(1 << 40), 1 << 40, n)
        v[rng.random(n) < 0.01] = np.iinfo(np.int64).max
        return v
    if t == D.GDF_DATE32:
        return rng.integers(-40000, 40000, n)
    if t == D.GDF_DATE64:
        return rng.integers(-4_000_000_000_000, 4_000_000_000_000, n)
    v = rng.standard_normal(n) * 1000
    special = rng.random(n)
    v[special < 0.01] = 0.0
    v[(special >= 0.01) & (special < 0.02)] = -0.0
    v[(special >= 0.02) & (special < 0.025)] = np.inf
    v[(special >= 0.025) & (special < 0.03)] = np.nan
    return v


def is_int_type(t):
    return t not in (D.GDF_FLOAT32, D.GDF_FLOAT64)


def random_program(rng, n_in, n_out, in_types, n_ops, transcendental=False):
    """A valid program whose last n_out ops write the output registers."""
    J = (D.GDF_INT32, 0)
    avail = list(range(n_in))
    kind = {i: (not is_int_type(in_types[i])) for i in range(n_in)}   # True = double register
    L, R_, O_, B, U, LS, RS = [], [], [], [], [], [], []
    next_tmp = n_in + n_out
    for k in range(n_ops):
        last = k >= n_ops - n_out
        out = (n_in + (k - (n_ops - n_out))) if last else next_tmp
        if not last:
            next_tmp += 1
        unary = rng.random() < 0.3
        if unary:
            cols = [i for i in avail if i < n_in]
            if transcendental and rng.random() < 0.6:
                op = TRANS_UN[rng.integers(len(TRANS_UN))]
                src = avail[rng.integers(len(avail))]
            else:
                op = EXACT_UN[rng.integers(len(EXACT_UN))]
                src = cols[rng.integers(len(cols))] if op in (D.BLZ_IS_NULL, D.BLZ_IS_NOT_NULL) else \
                    avail[rng.integers(len(avail))]
            L.append(src); R_.append(-1); B.append(D.GDF_INVALID_BINARY); U.append(op); LS.append(J); RS.append(J)
            kind[out] = False if op in (D.BLZ_NOT, D.BLZ_IS_NULL, D.BLZ_IS_NOT_NULL, D.BLZ_YEAR, D.BLZ_MONTH,
                                        D.BLZ_DAY, D.BLZ_HOUR, D.BLZ_MINUTE, D.BLZ_SECOND) and not kind.get(src) \
                else kind.get(src, False)
        else:
            op = EXACT_BIN[rng.integers(len(EXACT_BIN))]
            if op == D.GDF_COALESCE:
                cols = [i for i in avail if i < n_in]
                lsrc = cols[rng.integers(len(cols))]
            else:
                lsrc = avail[rng.integers(len(avail))] if rng.random() > 0.1 else -2
            r = rng.random()
            rsrc = avail[rng.integers(len(avail))] if r > 0.25 else (-2 if r > 0.03 else -3)
            if op in (D.GDF_DIV, D.GDF_MOD, D.GDF_FLOOR_DIV):
                lk = kind.get(lsrc, False) if lsrc >= 0 else False
                rk = kind.get(rsrc, False) if rsrc >= 0 else False
                if op == D.GDF_MOD or not (lk or rk):
                    rsrc = -2   # integer divisor: a nonzero literal (x/0 has no pinned GPU value)
            ls = J if lsrc != -2 else ((D.GDF_INT64, int(rng.integers(-9, 10))) if rng.random() < 0.6
                                       else (D.GDF_FLOAT64, float(rng.standard_normal() * 10)))
            if rsrc == -2:
                if op in (D.GDF_DIV, D.GDF_MOD, D.GDF_FLOOR_DIV):
                    v = int(rng.integers(1, 50)) * (1 if rng.random() < 0.5 else -1)
                    rs = (D.GDF_INT64, v) if rng.random() < 0.7 else (D.GDF_INT32, v)
                else:
                    rs = (D.GDF_INT64, int(rng.integers(-100, 100))) if rng.random() < 0.5 else \
                        (D.GDF_FLOAT64, float(rng.standard_normal() * 100))
            elif rsrc == -3:
                rs = (D.GDF_INT32, 0, False)
            else:
                rs = J
            L.append(lsrc); R_.append(rsrc); B.append(op); U.append(D.BLZ_INVALID_UNARY); LS.append(ls); RS.append(rs)
        O_.append(out)
        avail.append(out)
    return dict(left=L, right=R_, outputs=O_, final=[n_in + o for o in range(n_out)], ops=B, uops=U, lscalars=LS,
                rscalars=RS)


@pytest.mark.parametrize("seed", range(40))
def test_random_programs_exact(seed):
    rng = np.random.default_rng(1000 + seed)
    n_in = int(rng.integers(1, 6))
    n_out = int(rng.integers(1, 4))
    in_types = [IN_TYPES[rng.integers(len(IN_TYPES))] for _ in range(n_in)]
    out_types = [OUT_TYPES[rng.integers(len(OUT_TYPES))] for _ in range(n_out)]
    n = int(rng.choice([1, 5, 32, 33, 100, 257, 4096, 10_007]))
    spec = []
    for t in in_types:
        vals = rand_values(rng, t, n)
        nr = float(rng.choice([0.0, 0.1, 0.5]))
        spec.append((t, vals, (rng.random(n) >= nr) if rng.random() < 0.7 else None))
    prog = random_program(rng, n_in, n_out, in_types, int(rng.integers(n_out, n_out + 12)))
    try:
        dev, ora = H.run_program_both(spec, out_types, prog)
    except O.OracleError as e:
        pytest.skip(f"program rejected by the oracle: {e}")
    for k, (g, e) in enumerate(zip(dev, ora)):
        H.assert_columns_equal(g, e, what=f"seed {seed} output {k}", check_null_count=False)


@pytest.mark.parametrize("seed", range(10))
def test_random_programs_transcendental(seed):
    rng = np.random.default_rng(5000 + seed)
    n_in = int(rng.integers(1, 4))
    in_types = [D.GDF_FLOAT64 if rng.random() < 0.7 else D.GDF_INT32 for _ in range(n_in)]
    n = 4099
    spec = [(t, rng.uniform(-0.99, 0.99, n) if t == D.GDF_FLOAT64 else rng.integers(1, 9, n), None)
            for t in in_types]
    # a single transcendental op per output keeps the comparison within the per-op ulp bound
    ops = TRANS_UN
    op = ops[seed % len(ops)]
    prog = dict(left=[0], right=[-1], outputs=[n_in], final=[n_in], ops=[D.GDF_INVALID_BINARY], uops=[op],
                lscalars=[(D.GDF_INT32, 0)], rscalars=[(D.GDF_INT32, 0)])
    dev, ora = H.run_program_both(spec, [D.GDF_FLOAT64], prog)
    # COTAN is cos/sin: two rounded transcendentals and a division
    tol = 2 * H.ULP_TOL if op == D.BLZ_COTAN else H.ULP_TOL
    H.assert_columns_equal(dev[0], ora[0], tol_ulp=tol, check_null_count=False)


def test_pow_float_and_int():
    n = 3000
    rng = np.random.default_rng(77)
    spec = [(D.GDF_FLOAT64, rng.uniform(0.1, 3, n), None), (D.GDF_INT64, rng.integers(-3, 40, n), None),
            (D.GDF_INT64, rng.integers(-5, 5, n), None)]
    prog = dict(left=[0, 2], right=[1, 1], outputs=[3, 4], final=[3, 4], ops=[D.GDF_POW, D.GDF_POW],
                uops=[D.BLZ_INVALID_UNARY] * 2, lscalars=[(D.GDF_INT32, 0)] * 2, rscalars=[(D.GDF_INT32, 0)] * 2)
    dev, ora = H.run_program_both(spec, [D.GDF_FLOAT64, D.GDF_INT64], prog)
    H.assert_columns_equal(dev[0], ora[0], tol_ulp=H.ULP_TOL, check_null_count=False)
    H.assert_columns_equal(dev[1], ora[1], check_null_count=False)


# ---- alignment, materialize, errors -------------------------------------------------------------

def test_unaligned_column_views():
    spec = W.fused_project_program()
    n = 5003
    inputs = W.fused_project_host(n + 1, seed=12)
    dev_in = H.to_device(inputs)
    # shift every input by one element: buffers are no longer 16-byte aligned
    shifted = []
    for c in dev_in:
        s = R.Column(c.data[1:], None, c.dtype, size=n)
        shifted.append(s)
    ora_in = [O.make_column(v[1:], t) for t, v, _ in inputs]
    outs = [R.Column.empty(t, n, with_valid=False) for t in spec.output_dtypes]
    R.perform_operation(outs, shifted, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops,
                        spec.lscalars, spec.rscalars)
    eo = [O.alloc_column(t, n, with_valid=False) for t in spec.output_dtypes]
    O.perform_operation(eo, ora_in, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops,
                        [fe.Scalar(*s) for s in spec.lscalars], [fe.Scalar(*s) for s in spec.rscalars])
    for g, e in zip(outs, eo):
        H.assert_columns_equal(g, e, check_null_count=False)


@pytest.mark.parametrize("idx_type", [D.GDF_INT32, D.GDF_INT64])
def test_materialize_column(idx_type):
    n = 10_000
    rng = np.random.default_rng(3)
    for t, vals in ((D.GDF_FLOAT64, rng.standard_normal(n)), (D.GDF_INT8, rng.integers(-100, 100, n)),
                    (D.GDF_INT32, rng.integers(0, 1000, n))):
        valid = rng.random(n) < 0.8
        col = R.Column.from_numpy(vals, t, valid)
        idx = rng.integers(-1, n, 7777)
        got = R.materialize_column(col, R.Column.from_numpy(idx, idx_type))
        oc = O.make_column(vals, t, valid)
        exp = O.materialize_column(oc, idx.astype(np.int32))
        H.assert_columns_equal(got, exp)


def test_rejected_programs_raise():
    c = R.Column.from_numpy(np.arange(10), D.GDF_INT64)
    out = R.Column.empty(D.GDF_INT64, 10)
    with pytest.raises(R.RalError) as ei:
        # reads register 5 before anything writes it
        R.perform_operation([out], [c], [5], [0], [1], [1], [D.GDF_ADD], [D.BLZ_INVALID_UNARY],
                            [(D.GDF_INT32, 0)], [(D.GDF_INT32, 0)])
    assert ei.value.code == 2
    with pytest.raises(R.RalError):
        R.evaluate_expression([c], "LIKE($0, 'x')", out)


@pytest.mark.parametrize("n", [1, 31, 4095, 4096, 4097, 1_000_003])
def test_apply_boolean_mask(n):
    rng = np.random.default_rng(n)
    st = rng.integers(-3, 4, n).astype(np.int8)
    v = rng.random(n) < 0.9
    for valid in (v, None):
        col = R.Column.from_numpy(st, D.GDF_INT8, valid)
        got = R.apply_boolean_mask(col)
        exp = O.apply_boolean_mask(O.make_column(st, D.GDF_INT8, valid))
        assert got.size == len(exp)
        np.testing.assert_array_equal(got.to_numpy(), exp)


@pytest.mark.parametrize("n", [1, 100, 2047, 2048, 2049, 300_001])
def test_filter_project_mixed_outputs(n, filter_mode):
    """Evaluated and pass-through projections over a filter; masks, literals, IS NULL, COALESCE."""
    rng = np.random.default_rng(n + 7)
    spec = [(D.GDF_INT32, rng.integers(0, 100, n), rng.random(n) < 0.9),
            (D.GDF_FLOAT64, rng.standard_normal(n), rng.random(n) < 0.8),
            (D.GDF_INT64, rng.integers(-1000, 1000, n), None),
            (D.GDF_INT8, rng.integers(-5, 5, n), rng.random(n) < 0.7),
            (D.GDF_FLOAT32, rng.standard_normal(n).astype(np.float32), None)]
    filt = "LogicalFilter(condition=[OR(<($0, 30), >($2, 500))])"
    proj = ("LogicalProject(a=[$2], b=[*($1, 2.5)], c=[+($0, $3)], d=[$3], e=[IS NULL($1)], "
            "f=[CASE(IS NOT NULL($0), $0, -1)], g=[$4], h=[-($4, $1)])")
    got = R.filter_project(H.to_device(spec), filt, proj)
    ef = O.process_filter(H.to_oracle(spec), filt)
    ep = O.execute_project_plan(ef, proj)
    assert len(got) == len(ep)
    for k, (g, e) in enumerate(zip(got, ep)):
        H.assert_columns_equal(g, e, what=f"projection {k}")


def test_filter_on_double_and_date_predicates(filter_mode):
    n = 70_001
    rng = np.random.default_rng(70)
    spec = [(D.GDF_FLOAT64, rng.standard_normal(n), rng.random(n) < 0.95),
            (D.GDF_DATE32, rng.integers(0, 2400, n), None),
            (D.GDF_DATE64, rng.integers(0, 200 * 86400000, n).astype(np.int64), rng.random(n) < 0.9)]
    q = "LogicalFilter(condition=[AND(>($0, -0.5), =(EXTRACT(FLAG(MONTH), $1), 3), <(EXTRACT(FLAG(DAY), $2), 15))])"
    got = R.process_filter(H.to_device(spec), q)
    exp = O.process_filter(H.to_oracle(spec), q)
    for k, (g, e) in enumerate(zip(got, exp)):
        H.assert_columns_equal(g, e, what=f"column {k}")


def test_filter_unaligned_frame(filter_mode):
    n = 9_999
    rng = np.random.default_rng(5)
    base = [(D.GDF_INT32, rng.integers(0, 100, n + 1), None), (D.GDF_FLOAT64, rng.standard_normal(n + 1), None)]
    dev = H.to_device(base)
    shifted = [R.Column(c.data[1:], None, c.dtype, size=n) for c in dev]
    q = "LogicalFilter(condition=[<($0, 40)])"
    got = R.process_filter(shifted, q)
    exp = O.process_filter([O.make_column(v[1:], t) for t, v, _ in base], q)
    for g, e in zip(got, exp):
        H.assert_columns_equal(g, e)


def test_integer_division_by_zero_and_overflow_are_defined():
    """x / 0, x % 0, INT64_MIN / -1 and x % -1 are undefined in the reference; both sides define
    them the same way (0, 0, INT64_MIN, 0), so every kernel and the oracle agree bit for bit."""
    n = 4096
    rng = np.random.default_rng(77)
    a = rng.integers(-(1 << 62), 1 << 62, n, dtype=np.int64)
    b = rng.choice(np.array([0, -1, 1, 7, -3, np.iinfo(np.int64).min], dtype=np.int64), n)
    a[:64] = np.iinfo(np.int64).min
    b[:32] = -1
    spec = [(D.GDF_INT64, a, None), (D.GDF_INT64, b, (rng.random(n) > 0.1))]
    J = (D.GDF_INT32, 0)
    prog = dict(left=[0, 0, 0], right=[1, 1, 1], outputs=[2, 3, 4], final=[2, 3, 4],
                ops=[D.GDF_DIV, D.GDF_MOD, D.GDF_FLOOR_DIV], uops=[D.BLZ_INVALID_UNARY] * 3,
                lscalars=[J] * 3, rscalars=[J] * 3)
    dev, ora = H.run_program_both(spec, [D.GDF_INT64, D.GDF_INT64, D.GDF_INT64], prog)
    for k, (g, e) in enumerate(zip(dev, ora)):
        H.assert_columns_equal(g, e, what=f"output {k}", check_null_count=False)


@pytest.mark.parametrize("d", [0, 1, -1, 2, -2, 3, 7, -7, 10, 1000, -1000, 65537, 1 << 31, -(1 << 31), (1 << 32) + 1,
                               1 << 62, -(1 << 62), (1 << 63) - 1, -(1 << 63)])
def test_integer_division_by_literal(d):
    """Division and remainder by a literal run with a multiplier precomputed on the host (no
    division per row); every divisor class (0, +-1, powers of two, INT64_MIN, the largest) against
    the oracle, on int64, int32 and float64 dividends including the extremes."""
    n = 4096
    rng = np.random.default_rng(abs(d) % 1000 + 5)
    a = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, n, dtype=np.int64)
    a[:8] = [np.iinfo(np.int64).min, np.iinfo(np.int64).max, 0, 1, -1, d if d > np.iinfo(np.int64).min else 0, -7, 7]
    a[8:1000] >>= rng.integers(0, 63, 992)
    b = rng.integers(-(1 << 31), 1 << 31, n).astype(np.int32)
    x = rng.standard_normal(n) * 1e6
    spec = [(D.GDF_INT64, a, rng.random(n) > 0.1), (D.GDF_INT32, b, None), (D.GDF_FLOAT64, x, None)]
    J = (D.GDF_INT32, 0)
    L = (D.GDF_INT64, d)
    prog = dict(left=[0, 0, 0, 1, 1, 2], right=[-2] * 6, outputs=[3, 4, 5, 6, 7, 8], final=[3, 4, 5, 6, 7, 8],
                ops=[D.GDF_DIV, D.GDF_MOD, D.GDF_FLOOR_DIV, D.GDF_DIV, D.GDF_MOD, D.GDF_MOD],
                uops=[D.BLZ_INVALID_UNARY] * 6, lscalars=[J] * 6, rscalars=[L] * 6)
    dev, ora = H.run_program_both(spec, [D.GDF_INT64] * 6, prog)
    for k, (g, e) in enumerate(zip(dev, ora)):
        H.assert_columns_equal(g, e, what=f"output {k}, divisor {d}", check_null_count=False)


def test_nan_to_integer_is_int64_min_as_on_the_gpu():
    """MOD converts its operands with cvt.rzi.s64.f64, which turns a NaN into INT64_MIN; the
    oracle does the same (INT64_MIN % k, then stored through the float register)."""
    n = 1000
    x = np.full(n, np.nan)
    x[::3] = 2.5
    spec = [(D.GDF_FLOAT64, x, None), (D.GDF_INT64, np.arange(1, n + 1, dtype=np.int64), None)]
    J = (D.GDF_INT32, 0)
    prog = dict(left=[0], right=[1], outputs=[2], final=[2], ops=[D.GDF_MOD], uops=[D.BLZ_INVALID_UNARY],
                lscalars=[J], rscalars=[J])
    dev, ora = H.run_program_both(spec, [D.GDF_FLOAT64], prog)
    # row 2: INT64_MIN % 3 = -2
    assert ora[0].data[2] == -2.0
    H.assert_columns_equal(dev[0], ora[0], what="MOD of NaN", check_null_count=False)


@pytest.mark.parametrize("sel", [0.01, 0.5, 0.99])
def test_filter_project_workload_matches_oracle(sel, filter_mode):
    """The 200M-row fused filter + project workload's query, at 300k rows."""
    spec = W.fused_project_host(300_001, seed=8)
    got = R.filter_project(H.to_device(spec), W.filter_project_filter(sel), W.FILTER_PROJECT_PROJECT)
    ef = O.process_filter(H.to_oracle(spec), W.filter_project_filter(sel))
    ep = O.execute_project_plan(ef, W.FILTER_PROJECT_PROJECT)
    assert len(got) == len(ep) == 3
    for k, (g, e) in enumerate(zip(got, ep)):
        H.assert_columns_equal(g, e, what=f"projection {k}")


@pytest.mark.parametrize("tune", ["D=0", "K=2,B=5", "P=1", "J=32,B=4", "D=1,J=4"])
def test_filter_project_launch_variants_match_oracle(tune, monkeypatch):
    """Every pass-2 form of the fused filter (slice-wise; kept-row list one or two steps at a time,
    with or without the look-back prefetch; other chunk sizes) gives the oracle's bits."""
    monkeypatch.setenv("RAL_FILTER_TUNE", tune)
    n = 200_003
    rng = np.random.default_rng(91)
    spec = [(D.GDF_INT32, rng.integers(0, 100, n), rng.random(n) < 0.9),
            (D.GDF_FLOAT64, rng.standard_normal(n), rng.random(n) < 0.8),
            (D.GDF_INT64, rng.integers(-1000, 1000, n), None),
            (D.GDF_INT8, rng.integers(-5, 5, n), rng.random(n) < 0.7)]
    filt = "LogicalFilter(condition=[OR(<($0, 45), >($2, 700))])"
    proj = ("LogicalProject(a=[$2], b=[*($1, 2.5)], c=[+($0, $3)], d=[$3], e=[IS NULL($1)], "
            "f=[CASE(IS NOT NULL($0), $0, -1)], g=[FLOOR(/($1, 3))], h=[MOD($2, +($0, 1))])")
    got = R.filter_project(H.to_device(spec), filt, proj)
    ef = O.process_filter(H.to_oracle(spec), filt)
    ep = O.execute_project_plan(ef, proj)
    for k, (g, e) in enumerate(zip(got, ep)):
        H.assert_columns_equal(g, e, what=f"{tune}: projection {k}")


def test_multiply_by_comparison_and_abs_on_special_values():
    """A double times a 0/1 comparison result skips the FP64 multiply and ABS may fold into its
    consumer; infinities, NaN, signed zeros and subnormals give the multiply's results."""
    specials = np.array([0.0, -0.0, 1.5, -2.25, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 1e308, -1e-310],
                        dtype=np.float64)
    n = len(specials) * 4
    x = np.tile(specials, 4)
    b = np.repeat(np.array([-1, 0, 1, 7], dtype=np.int64), len(specials))
    spec = [(D.GDF_FLOAT64, x, None), (D.GDF_INT64, b, None)]
    J, I64 = (D.GDF_INT32, 0), (D.GDF_INT64, 0)
    # registers: $0 = x, $1 = b, outputs 2..5, temporaries from 6
    # c = b > 0 (6); m = c * x (5); a = |x| (7); s = a + m (2); d = |x| stored (3); z = m - a (4)
    prog = dict(left=[1, 6, 0, 7, 0, 5], right=[-2, 0, -1, 5, -1, 7], outputs=[6, 5, 7, 2, 3, 4],
                final=[2, 3, 4, 5],
                ops=[D.GDF_GREATER, D.GDF_MUL, D.GDF_INVALID_BINARY, D.GDF_ADD, D.GDF_INVALID_BINARY, D.GDF_SUB],
                uops=[D.BLZ_INVALID_UNARY, D.BLZ_INVALID_UNARY, D.BLZ_ABS, D.BLZ_INVALID_UNARY, D.BLZ_ABS,
                      D.BLZ_INVALID_UNARY],
                lscalars=[J] * 6, rscalars=[I64, J, J, J, J, J])
    dev, ora = H.run_program_both(spec, [D.GDF_FLOAT64] * 4, prog)
    for k, (g, e) in enumerate(zip(dev, ora)):
        H.assert_columns_equal(g, e, what=f"output {k}", check_null_count=False)


@pytest.mark.parametrize("pinned", [True, False])
def test_host_buffer_evaluation_matches_device_columns(pinned):
    """ral_perform_operation_host streams host columns through the GPU in chunks (here three
    full chunks and a partial one, on three streams) and gives the device call's bits and null
    counts; page-locked or not."""
    n = 3_000_123
    spec = W.fused_project_program()
    host = W.fused_project_host(n, seed=5)
    dev_in = H.to_device(host)
    dev_out = [R.Column.empty(t, n) for t in spec.output_dtypes]
    R.perform_operation(dev_out, dev_in, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops,
                        spec.lscalars, spec.rscalars)

    def host_copy(t):
        t = t.cpu()
        return t.pin_memory() if pinned else t

    hin = [R.Column(host_copy(c.data), host_copy(c.valid), c.dtype, size=n, null_count=c.null_count) for c in dev_in]
    hout = []
    for t in spec.output_dtypes:
        c = R.Column.empty(t, n, device="cpu")
        hout.append(R.Column(host_copy(c.data), host_copy(c.valid), t, size=n))
    R.perform_operation_host(hout, hin, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops,
                             spec.lscalars, spec.rscalars, chunk_rows=1_000_000)
    for k, (g, e) in enumerate(zip(hout, dev_out)):
        ev = e.valid_bools()
        assert np.array_equal(g.valid_bools(), ev), f"output {k}: masks differ"
        assert np.array_equal(g.to_numpy()[ev].view(np.uint8), e.to_numpy()[ev].view(np.uint8)), f"output {k}: data"
        assert g.null_count == int((~ev).sum())
