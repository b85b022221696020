"""Shared helpers: build matching oracle (host) and library (device) columns and compare results.

Comparison rules used by every parity test:
  * validity bits are compared for every row < n;
  * data is compared where the expected validity bit is set (the reference
    computes data for null rows too, from whatever the null slots hold);
  * integer and exactly-rounded float results are compared bit for bit, with
    one exception: any NaN equals any NaN (the GPU's canonical NaN and the
    x86 default NaN differ only in payload);
  * transcendental results (sin, cos, tan, asin, acos, atan, log, log10,
    pow) are compared within 2 ulp (ULP_TOL), as CUDA's and libm's
    implementations differ in the last bits.
"""
from __future__ import annotations

import numpy as np

import oracle as O
import ralgpu as R

ULP_TOL = 2


def to_device(spec):
    """spec: [(dtype, values, valid_bools or None)] -> [ralgpu.Column]"""
    return [R.Column.from_numpy(v, t, m) for t, v, m in spec]


def to_oracle(spec):
    return [O.make_column(v, t, m) for t, v, m in spec]


def _bits(a: np.ndarray) -> np.ndarray:
    if a.dtype == np.float64:
        return a.view(np.int64)
    if a.dtype == np.float32:
        return a.view(np.int32)
    return a


def ulp_distance(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Distance in units in the last place between same-typed float arrays."""
    def ordered(x):
        if x.dtype == np.float64:
            v = x.view(np.int64)
            return np.where(v < 0, -(v & np.int64(0x7FFFFFFFFFFFFFFF)), v)
        v = x.view(np.int32).astype(np.int64)
        return np.where(v < 0, -(v & 0x7FFFFFFF), v)
    return np.abs(ordered(a) - ordered(b))


def assert_data_equal(got: np.ndarray, exp: np.ndarray, mask: np.ndarray, tol_ulp: int = 0, what: str = ""):
    g = got[mask]
    e = exp[mask]
    if g.dtype.kind == "f":
        gn, en = np.isnan(g), np.isnan(e)
        assert np.array_equal(gn, en), f"{what}: NaN positions differ"
        g, e = g[~gn], e[~en]
        if tol_ulp:
            d = ulp_distance(g, e)
            bad = np.nonzero(d > tol_ulp)[0]
            assert bad.size == 0, f"{what}: {bad.size} values beyond {tol_ulp} ulp, first {g[bad[:3]]} vs {e[bad[:3]]}"
            return
        gb, eb = _bits(g), _bits(e)
        bad = np.nonzero(gb != eb)[0]
        # +0.0 and -0.0 are different bit patterns and the reference distinguishes them too
        assert bad.size == 0, f"{what}: {bad.size} mismatches, first rows {np.nonzero(mask)[0][bad[:5]]}: " \
                              f"{g[bad[:5]]} vs {e[bad[:5]]}"
    else:
        bad = np.nonzero(g != e)[0]
        assert bad.size == 0, f"{what}: {bad.size} mismatches, first {g[bad[:5]]} vs {e[bad[:5]]}"


def assert_columns_equal(got: R.Column, exp: O.OColumn, tol_ulp: int = 0, what: str = "", check_null_count=True):
    assert got.size == exp.size, f"{what}: size {got.size} != {exp.size}"
    gv = got.valid_bools()
    ev = exp.valid_bools()
    assert (got.valid is None) == (exp.valid is None), f"{what}: validity presence differs"
    bad = np.nonzero(gv != ev)[0]
    assert bad.size == 0, f"{what}: {bad.size} validity mismatches, first rows {bad[:5]}"
    assert_data_equal(got.to_numpy(), exp.data[:exp.size], ev, tol_ulp, what)
    if check_null_count:
        assert got.null_count == exp.null_count, f"{what}: null_count {got.null_count} != {exp.null_count}"


def run_program_both(spec_inputs, out_dtypes, prog, out_valid=True, nthreads=8):
    """Runs a program (dict with left/right/outputs/final/ops/uops/lscalars/rscalars) on both sides."""
    dev_in = to_device(spec_inputs)
    ora_in = to_oracle(spec_inputs)
    n = dev_in[0].size
    dev_out = [R.Column.empty(t, n, with_valid=out_valid) for t in out_dtypes]
    ora_out = [O.alloc_column(t, n, with_valid=out_valid) for t in out_dtypes]
    R.perform_operation(dev_out, dev_in, prog["left"], prog["right"], prog["outputs"], prog["final"], prog["ops"],
                        prog["uops"], prog["lscalars"], prog["rscalars"])
    from oracle import frontend as fe
    O.perform_operation(ora_out, ora_in, prog["left"], prog["right"], prog["outputs"], prog["final"], prog["ops"],
                        prog["uops"], [fe.Scalar(*s) if isinstance(s, tuple) else fe.Scalar(s.dtype, s.value, s.is_valid)
                                       for s in prog["lscalars"]],
                        [fe.Scalar(*s) if isinstance(s, tuple) else fe.Scalar(s.dtype, s.value, s.is_valid)
                         for s in prog["rscalars"]], nthreads=nthreads)
    return dev_out, ora_out
