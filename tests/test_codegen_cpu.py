"""Generated kernels compile with NVRTC for sm_103a (no GPU needed) and do not spill."""
import re

import pytest

import ralgpu
from ralgpu import dtypes as D
from ralgpu import workloads as W


def compile_spec(spec: W.ProgramSpec, nullable=True):
    src, log = ralgpu.debug_program_source(
        spec.input_dtypes, [1 if nullable else 0] * len(spec.input_dtypes), spec.output_dtypes,
        [1 if nullable else 0] * len(spec.output_dtypes), spec.left, spec.right, spec.outputs, spec.final,
        spec.ops, spec.uops, spec.lscalars, spec.rscalars, compile=True)
    return src, log


def spills(log: str) -> int:
    total = 0
    for m in re.finditer(r"(\d+) bytes spill stores", log):
        total += int(m.group(1))
    return total


def test_fused_project_kernel_compiles():
    src, log = compile_spec(W.fused_project_program())
    assert "__ddiv_rn" in src and "ral_modi" in src and "floor(" in src
    assert "ral_eval_" in src
    assert spills(log) == 0, log
    assert "registers" in log


def test_fused_project_kernel_without_masks_compiles():
    src, log = compile_spec(W.fused_project_program(), nullable=False)
    assert "ral_vword" not in src
    assert spills(log) == 0, log


def _all_ops_program():
    """Every binary and unary operator over int32 / int64 / float32 / float64 / date32 / date64 inputs."""
    ins = [D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64, D.GDF_DATE32, D.GDF_DATE64]
    n_in = len(ins)
    L, R, O, B, U = [], [], [], [], []
    outs = []
    binops = [D.GDF_ADD, D.GDF_SUB, D.GDF_MUL, D.GDF_DIV, D.GDF_FLOOR_DIV, D.GDF_MOD, D.GDF_POW, D.GDF_EQUAL,
              D.GDF_NOT_EQUAL, D.GDF_LESS, D.GDF_GREATER, D.GDF_LESS_EQUAL, D.GDF_GREATER_EQUAL, D.GDF_COALESCE]
    unops = [D.BLZ_FLOOR, D.BLZ_CEIL, D.BLZ_SIN, D.BLZ_COS, D.BLZ_ASIN, D.BLZ_ACOS, D.BLZ_TAN, D.BLZ_COTAN,
             D.BLZ_ATAN, D.BLZ_ABS, D.BLZ_NOT, D.BLZ_LN, D.BLZ_LOG, D.BLZ_YEAR, D.BLZ_MONTH, D.BLZ_DAY,
             D.BLZ_HOUR, D.BLZ_MINUTE, D.BLZ_SECOND, D.BLZ_IS_NULL, D.BLZ_IS_NOT_NULL, D.BLZ_INVALID_UNARY]
    n_out = len(binops) + len(unops)
    k = 0
    for i, op in enumerate(binops):
        L.append(i % n_in if op != D.GDF_COALESCE else 1)
        R.append((i + 3) % n_in)
        O.append(n_in + k); B.append(op); U.append(D.BLZ_INVALID_UNARY); k += 1
    for i, op in enumerate(unops):
        L.append(i % n_in); R.append(-1); O.append(n_in + k); B.append(D.GDF_INVALID_BINARY); U.append(op); k += 1
    out_types = [D.GDF_FLOAT64 if j % 2 else D.GDF_INT64 for j in range(n_out)]
    J = (D.GDF_INT32, 0)
    return W.ProgramSpec(ins, out_types, L, R, O, [n_in + j for j in range(n_out)], B, U, [J] * len(L),
                         [J] * len(L))


def test_every_operator_compiles():
    src, log = compile_spec(_all_ops_program())
    for fn in ("ral_powi", "pow(", "sin(", "log10(", "ral_year32", "ral_hour64", "ral_month64"):
        assert fn in src, fn


@pytest.mark.parametrize("nullable", [True, False])
def test_plain_vm_filter_program_compiles(nullable):
    from oracle import frontend as fe
    res = fe.plan_evaluate_expression(4, fe.get_condition_expression(W.PLAIN_VM_FILTER))
    plan, cols = res[1], res[2]
    src, log = ralgpu.debug_program_source(
        [W.PLAIN_VM_DTYPES[c] for c in cols], [1 if nullable else 0] * len(cols), [D.GDF_INT8], [1],
        plan.left, plan.right, plan.outputs, plan.final_output_positions, plan.operators, plan.unary_operators,
        [ralgpu.Scalar(s.dtype, s.value, s.is_valid) for s in plan.left_scalars],
        [ralgpu.Scalar(s.dtype, s.value, s.is_valid) for s in plan.right_scalars], compile=True)
    assert spills(log) == 0, log
    # MOD($0, 7): the remainder by a literal uses the host's precomputed divider
    import re
    assert re.search(r"ral_sf_modc\((?!long long)", src) and not re.search(r"ral_modi\((?!ral_i64 a)", src)


FILTER_CASES = [
    ("filter_gather nullable", W.FILTER_GATHER_DTYPES, [1] * 6, W.filter_gather_query(0.5), None),
    ("filter_gather null-free", W.FILTER_GATHER_DTYPES, [0] * 6, W.filter_gather_query(0.01), None),
    ("plain_vm filter+project", W.PLAIN_VM_DTYPES, [0, 1, 0, 0], W.PLAIN_VM_FILTER, W.PLAIN_VM_PROJECT),
    ("bare column stencil", [D.GDF_INT8, D.GDF_BOOL8, D.GDF_FLOAT64], [1, 0, 1], "LogicalFilter(condition=[$1])",
     None),
    ("is null + coalesce projection", [D.GDF_INT32, D.GDF_FLOAT64, D.GDF_INT64], [1, 1, 0],
     "LogicalFilter(condition=[AND(IS NULL($0), >($2, 5))])",
     "LogicalProject(a=[$2], b=[CASE(IS NOT NULL($0), $0, -1)], c=[IS NULL($1)], d=[*($1, 2.5)])"),
]


@pytest.mark.parametrize("tune", ["", "S=1", "J=8,U=2,T=128,B=4", "J=64,U=8,T=512,B=1,S=1", "P=8", "P=4,J=16",
                                  "D=1", "D=0", "D=1,J=8,T=128", "K=2,B=5", "P=1,K=2,B=4", "R=1", "R=3,J=4",
                                  "R=2,J=2,T=128", "R=4,D=0"])
@pytest.mark.parametrize("case", FILTER_CASES, ids=[c[0] for c in FILTER_CASES])
def test_filter_kernels_compile(case, tune, monkeypatch):
    _, dtypes, nullable, fq, pq = case
    monkeypatch.setenv("RAL_FILTER_TUNE", tune)
    src, log = ralgpu.debug_filter_source(dtypes, nullable, fq, pq, compile=True)
    assert "ral_filter_" in src and "ral_lookback" in src
    assert spills(log) <= 64, log


def test_dense_pass_two_is_the_default_and_fits_shared_memory(monkeypatch):
    """Pass 2 walks the kept-row list by default, with a projection or gathers only; D=0 selects
    the slice-wise pass; a shape whose per-block lists would not fit static shared memory falls
    back to it."""
    monkeypatch.delenv("RAL_FILTER_TUNE", raising=False)
    p = W.fused_project_program()
    src, _ = ralgpu.debug_filter_source(p.input_dtypes, [1] * 5, W.filter_project_filter(0.5),
                                        W.FILTER_PROJECT_PROJECT)
    assert "s_lst[actA ? kA : k0]" in src and "kbw[" not in src
    src, _ = ralgpu.debug_filter_source(W.FILTER_GATHER_DTYPES, [1] * 6, W.filter_gather_query(0.5), None)
    assert "s_lst[actA ? kA : k0]" in src and "kbw[" not in src
    monkeypatch.setenv("RAL_FILTER_TUNE", "D=0")
    src, _ = ralgpu.debug_filter_source(W.FILTER_GATHER_DTYPES, [1] * 6, W.filter_gather_query(0.5), None)
    assert "s_lst" not in src and "kbw[" in src
    monkeypatch.setenv("RAL_FILTER_TUNE", "J=64,T=512,B=1")
    src, log = ralgpu.debug_filter_source(p.input_dtypes, [1] * 5, W.filter_project_filter(0.5),
                                          W.FILTER_PROJECT_PROJECT, compile=True)
    assert "s_lst" not in src and "kbw[" in src and spills(log) <= 64


def test_projection_filter_pipelines_two_chunks_per_warp(monkeypatch):
    """With a projection the kernel evaluates the next chunk's predicate before the look-back of
    the last one (keep bits as mask words, two chunks per warp); a chunk size with more than 32
    mask words falls back to one chunk at a time."""
    monkeypatch.delenv("RAL_FILTER_TUNE", raising=False)
    p = W.fused_project_program()
    src, log = ralgpu.debug_filter_source(p.input_dtypes, [1] * 5, W.filter_project_filter(0.5),
                                          W.FILTER_PROJECT_PROJECT, compile=True)
    assert "ral_lookback_publish(status, chunk, total)" in src and "chunkA" in src and spills(log) == 0
    monkeypatch.setenv("RAL_FILTER_TUNE", "J=32,B=4")
    src, log = ralgpu.debug_filter_source(p.input_dtypes, [1] * 5, W.filter_project_filter(0.5),
                                          W.FILTER_PROJECT_PROJECT, compile=True)
    assert "chunkA" not in src and "s_lst[actA ? kA : k0]" in src and spills(log) == 0


def _registers(log: str) -> int:
    m = re.findall(r"Used (\d+) registers", log)
    return max(int(x) for x in m) if m else 0


def test_default_shapes_keep_their_occupancy():
    """The measured defaults rely on resident warps: the 12-op projection as two 512-thread blocks
    per SM (at most 64 registers) and the fused filter + project as five 256-thread blocks (at most
    51), both without spills."""
    p = W.fused_project_program()
    src, log = compile_spec(p)
    assert "#define RAL_THREADS 512" in src and "__launch_bounds__(RAL_THREADS, 2)" in src
    assert spills(log) == 0 and _registers(log) <= 64, log
    src, log = ralgpu.debug_filter_source(p.input_dtypes, [1] * 5, W.filter_project_filter(0.5),
                                          W.FILTER_PROJECT_PROJECT, compile=True)
    assert "__launch_bounds__(RAL_THREADS, 5)" in src
    assert spills(log) == 0 and _registers(log) <= 51, log


AGG_DTYPES = [4, 4, 6, 6, 3, 5, 1, 2]   # int64, int64, float64, float64, int32, float32, int8, int16


@pytest.mark.parametrize("q", range(3))
def test_aggregate_kernels_compile_for_sm103a(q):
    """The fused aggregate kernels of the GPU test plans compile with NVRTC (no GPU needed)."""
    from test_gpu_aggregate import QUERIES
    src, log = ralgpu.debug_aggregate_source(AGG_DTYPES, [1, 1, 1, 1, 1, 0, 1, 0], [5, 5, 5, 5, 5, 0, 9, 0],
                                             QUERIES[q], compile=True)
    assert "ral_agg_" in src
    assert "error" not in log.lower()


def test_aggregate_count_only_needs_no_kernel_and_group_by_is_rejected():
    src, _ = ralgpu.debug_aggregate_source([3], [1], [2], "LogicalAggregate(group=[{}], EXPR$0=[COUNT()])")
    assert src == ""
    with pytest.raises(ralgpu.RalError, match="GROUP BY"):
        ralgpu.debug_aggregate_source([3, 4], [0, 0], [0, 0],
                                      "LogicalAggregate(group=[{0}], EXPR$0=[SUM($1)])")
    with pytest.raises(ralgpu.RalError):
        ralgpu.debug_aggregate_source([3], [0], [0], "LogicalAggregate(group=[{}], EXPR$0=[STDDEV($0)])")


def test_aggregate_plan_matches_the_oracle_parse():
    """Library and oracle split a LogicalAggregate the same way (names, operators, inputs)."""
    from oracle import frontend as fe
    q = ("LogicalAggregate(group=[{}], EXPR$0=[COUNT()], s=[SUM(*($0, -(1, $1)))], EXPR$2=[AVG($1)], "
         "m=[MIN(CAST($0):DOUBLE)], x=[MAX(+($0, 1))])")
    groups, aggs = fe.parse_aggregate(q)
    assert groups == [] and [a[1] for a in aggs] == [fe.GDF_COUNT, fe.GDF_SUM, fe.GDF_AVG, fe.GDF_MIN, fe.GDF_MAX]
    src, _ = ralgpu.debug_aggregate_source([4, 6], [0, 0], [0, 0], q, compile=False)
    # SUM, AVG, MIN and MAX each fold one slot; COUNT() needs none
    assert src.count("acc3 =") >= 1 and "acc4" not in src


def test_grid_mode_replaces_the_look_back(monkeypatch):
    """R=K: each warp owns K consecutive chunks, pass 1 of all of them, one grid barrier, then pass
    2 at offsets summed from block, warp and chunk counts; the kernel zeroes the output masks and
    valid counts itself.  Shapes without the mask-word pass 1 (D=0) keep the look-back."""
    p = W.fused_project_program()
    monkeypatch.setenv("RAL_FILTER_TUNE", "R=2")
    src, log = ralgpu.debug_filter_source(p.input_dtypes, [1] * 5, W.filter_project_filter(0.5),
                                          W.FILTER_PROJECT_PROJECT, compile=True)
    body = src[src.index("extern \"C\" __global__"):]
    assert "ral_grid_barrier(scratch, RAL_EPOCH + gridDim.x, scratch + 1)" in body
    assert "ral_lookback" not in body and "atomicAdd((unsigned int*)scratch" not in body
    assert "#define RAL_K 2" in src and spills(log) <= 64
    monkeypatch.setenv("RAL_FILTER_TUNE", "R=2,D=0")
    src, _ = ralgpu.debug_filter_source(p.input_dtypes, [1] * 5, W.filter_project_filter(0.5),
                                        W.FILTER_PROJECT_PROJECT)
    body = src[src.index("extern \"C\" __global__"):]
    assert "ral_grid_barrier" not in body and "ral_lookback" in body


@pytest.mark.parametrize("fq", [None, "LogicalFilter(condition=[>($2, 25)])",
                                "LogicalFilter(condition=[OR(IS NULL($3), <($4, 0.03))])",
                                "LogicalFilter(condition=[AND(>=($6, 1995-01-01), <($6, 1996-01-01 00:00:00))])"])
def test_text_scan_kernels_compile(fq):
    src, log = ralgpu.debug_text_scan_source(W.TEXT_DTYPES, list(range(8)), fq, compile=True)
    assert "ral_textscan_" in src and "ral_tx_parse_double" in src
    assert spills(log) == 0, log
