"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/ral_oracle.cpp into oracle/_build/libral_oracle.so with
-ffp-contract=off so that x*y+z is never fused (the GPU kernels are built with
--fmad=false for the same reason).  The reference itself cannot be compiled
here (it needs cudf, RMM, NVStrings and blazingdb-io headers and a GPU), so
there is no oracle/_ref build.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ral_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "libral_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-o", OUT + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
