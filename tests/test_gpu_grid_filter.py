"""Fused filters in grid mode: synchronous calls of at most 8Mi rows run as one cooperative launch
whose warps own fixed chunks, with one grid barrier between the predicate pass and the output pass
in place of the look-back.  Every output row is compared with the oracle (the benchmark's chunked
checker) and with the look-back kernel (RAL_FILTER_TUNE=R=0), across sizes that end inside a chunk,
a warp's chunks and a block, and on either side of the 8Mi-row limit."""
import numpy as np
import pytest

import bench
import ralgpu as R

pytestmark = pytest.mark.gpu


def _run(ctx):
    import torch
    ctx["step"](torch.cuda.current_stream())
    torch.cuda.synchronize()


def _outputs(ctx):
    n = ctx["nout"].value
    res = []
    for o in ctx["outs"]:
        v = o.data[:n].cpu().numpy().copy()
        m = None
        if o.valid is not None:
            m = o.valid[: (n + 31) // 32 * 4].cpu().numpy().view(np.uint32).copy()
            if n % 32:
                m[-1] &= (1 << (n % 32)) - 1
        res.append((v, m))
    return n, res


@pytest.mark.parametrize("workload,n,sel", [
    ("plain_vm", 1_000_000, None),
    ("plain_vm", 129, None),
    ("filter_project", 1_000_003, 0.5),
    ("filter_project", 4_000_037, 0.99),
    ("filter_gather", 3_000_017, 0.01),
    ("filter_gather", 8_388_608, 0.5),
])
def test_grid_mode_matches_the_oracle_and_the_look_back(workload, n, sel, monkeypatch):
    monkeypatch.delenv("RAL_FILTER_TUNE", raising=False)
    ctx = bench.filter_setup(workload, n, sel or 0.5, "cuda")
    g0 = R.filter_grid_launches()
    _run(ctx)
    assert R.filter_grid_launches() == g0 + 1, "the call did not run in grid mode"
    res = bench.parity_check(workload, ctx, sel or 0.5)
    assert res["mismatches"] == 0, res
    n_grid, out_grid = _outputs(ctx)
    _run(ctx)                        # a second call: the barrier counter continues from the first
    assert _outputs(ctx)[0] == n_grid
    monkeypatch.setenv("RAL_FILTER_TUNE", "R=0")
    _run(ctx)
    assert R.filter_grid_launches() == g0 + 2
    n_lb, out_lb = _outputs(ctx)
    assert n_lb == n_grid
    for k, ((a, ma), (b, mb)) in enumerate(zip(out_grid, out_lb)):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"output {k} data"
        assert (ma is None) == (mb is None) and (ma is None or np.array_equal(ma, mb)), f"output {k} mask"


def test_above_the_limit_the_look_back_runs(monkeypatch):
    monkeypatch.delenv("RAL_FILTER_TUNE", raising=False)
    ctx = bench.filter_setup("filter_gather", 8_388_609, 0.5, "cuda")
    g0 = R.filter_grid_launches()
    _run(ctx)
    assert R.filter_grid_launches() == g0
    res = bench.parity_check("filter_gather", ctx, 0.5)
    assert res["mismatches"] == 0, res


def test_forced_chunks_per_warp_and_sizes_in_turn(monkeypatch):
    """R=K forces K chunks per warp (fewer blocks, each warp several chunks); calls of different
    sizes in turn keep the barrier counter consistent."""
    monkeypatch.setenv("RAL_FILTER_TUNE", "R=5")
    for n in (70_001, 2_500_000, 1, 33, 600_000):
        ctx = bench.filter_setup("filter_project", n, 0.5, "cuda")
        _run(ctx)
        res = bench.parity_check("filter_project", ctx, 0.5)
        assert res["mismatches"] == 0, (n, res)
