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
"""
from __future__ import annotations

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
