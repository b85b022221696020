"""Batched execution, host side: the program mix plans, and the batch kernel compiles with
NVRTC for sm_103a (no GPU needed: column descriptors point at host buffers that are never read)."""
import re

import numpy as np

import ralgpu
from ralgpu import workloads as W


def test_batched_mix_is_deterministic_and_plans():
    a, b = W.batched_mix(64), W.batched_mix(64)
    assert [t.project for t in a] == [t.project for t in b]
    for t in a:
        assert 1e3 <= t.rows <= 5e7
        assert 2 <= len(t.dtypes) <= 8
        assert all(0.0 <= r <= 0.2 for r in t.null_rates)
        pp = ralgpu.parse_project_plan(t.dtypes, t.project)
        assert len(pp["operators"]) == t.n_ops
        assert 4 <= t.n_ops <= 48
        n_in = len(pp["input_columns"])
        assert pp["final_output_positions"] == [n_in + k for k in range(len(pp["evaluated_dtypes"]))]


def test_parse_project_plan_matches_add_expression_to_plan():
    frame = [ralgpu.dtypes.GDF_INT64, ralgpu.dtypes.GDF_FLOAT64, ralgpu.dtypes.GDF_INT32]
    pp = ralgpu.parse_project_plan(frame, "LogicalProject(a=[$0], b=[+(*($1, 2), $2)], c=[<($2, 5)])")
    # the program reads $1 and $2 only (dense inputs 0, 1); two evaluated expressions
    assert pp["input_columns"] == [1, 2]
    assert pp["evaluated_dtypes"] == [ralgpu.dtypes.GDF_FLOAT64, ralgpu.dtypes.GDF_INT8]
    first = ralgpu.add_expression_to_plan("+(*($1, 2), $2)", 0, 2, 2, [-1, 0, 1])
    assert pp["operators"][:len(first["operators"])] == first["operators"]
    assert pp["left"][:len(first["left"])] == first["left"]


def _fake_batch(mix, rows=1000):
    b = ralgpu.Batch()
    for t in mix:
        pp = ralgpu.parse_project_plan(t.dtypes, t.project)
        ins = [ralgpu.Column.empty(t.dtypes[c], rows, with_valid=t.null_rates[c] > 0, device="cpu")
               for c in pp["input_columns"]]
        for c in ins:
            c.null_count = 1 if c.valid is not None else 0
        outs = [ralgpu.Column.empty(dt, rows, with_valid=True, device="cpu") for dt in pp["evaluated_dtypes"]]
        b.add(outs, ins, pp["left"], pp["right"], pp["outputs"], pp["final_output_positions"], pp["operators"],
              pp["unary_operators"], pp["left_scalars"], pp["right_scalars"])
    return b


def test_batch_items_compile_and_link(tmp_path, monkeypatch):
    monkeypatch.setenv("RAL_JIT_CACHE_DIR", str(tmp_path))   # compile afresh, so ptxas logs exist
    mix = W.batched_mix(24, seed=7)
    b = _fake_batch(mix)
    assert b.info()["programs"] == 24
    src, log = b.debug_source(compile=True)
    assert src.count('extern "C" __device__ __noinline__ void ral_item_') == 24
    assert "atomicAdd(counter" in src and "case 23:" in src
    # item functions are capped at 96 registers (occupancy of the linked kernel); programs with
    # FP64 transcendentals may spill a little to local memory, never by kilobytes
    frames = [int(m) for m in re.findall(r"(\d+) bytes stack frame", log)]
    assert frames and max(frames) < 1024, log[-2000:]
    b.close()


def test_batch_rejects_mismatched_columns():
    mix = W.batched_mix(1, seed=3)
    t = mix[0]
    pp = ralgpu.parse_project_plan(t.dtypes, t.project)
    ins = [ralgpu.Column.empty(t.dtypes[c], 100, with_valid=False, device="cpu") for c in pp["input_columns"]]
    outs = [ralgpu.Column.empty(dt, 50, with_valid=True, device="cpu") for dt in pp["evaluated_dtypes"]]
    b = ralgpu.Batch()
    try:
        b.add(outs, ins, pp["left"], pp["right"], pp["outputs"], pp["final_output_positions"], pp["operators"],
              pp["unary_operators"], pp["left_scalars"], pp["right_scalars"])
    except ralgpu.RalError as e:
        assert e.code == 1 and "shorter" in str(e)
    else:
        raise AssertionError("short output accepted")
    finally:
        b.close()


def test_tune_keys_group_programs():
    mix = W.batched_mix(256)
    keys = set()
    for t in mix:
        pp = ralgpu.parse_project_plan(t.dtypes, t.project)
        ins = [ralgpu.Column.empty(t.dtypes[c], 10, with_valid=t.null_rates[c] > 0, device="cpu")
               for c in pp["input_columns"]]
        outs = [ralgpu.Column.empty(dt, 10, with_valid=True, device="cpu") for dt in pp["evaluated_dtypes"]]
        keys.add(ralgpu.batch_tune_key(outs, ins, pp["left"], pp["right"], pp["outputs"],
                                       pp["final_output_positions"], pp["operators"], pp["unary_operators"],
                                       pp["left_scalars"], pp["right_scalars"]))
    # a few dozen keys: the autotuner times one program per key, not every program
    assert 4 <= len(keys) <= 60, keys
    assert all(k.startswith("G") and ":ops" in k and ":f64" in k and ":in" in k for k in keys)
