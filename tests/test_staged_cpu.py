"""The staged (bulk-copy) eval kernels compile for sm_103a without a GPU.

Staging is a launch shape of the eval kernel (RAL_EVAL_TUNE key M = stages per warp); the shape is
read once per process, so each case runs in a subprocess."""
import json
import os
import subprocess
import sys

import pytest

from conftest import PKG, ROOT

SCRIPT = r"""
import json, sys
sys.path.insert(0, %r); sys.path.insert(0, %r)
import ralgpu as R
from ralgpu import workloads as W
spec = W.fused_project_program()
src, log = R.debug_program_source(spec.input_dtypes, [1] * 5, spec.output_dtypes, [1] * 3, spec.left, spec.right,
                                  spec.outputs, spec.final, spec.ops, spec.uops, spec.lscalars, spec.rscalars,
                                  compile=True)
k = src[src.find("extern \"C\""):]
print(json.dumps({"bulk": k.count("ral_bulk_g2s("), "wait": "ral_mbar_wait(" in k, "log": log}))
"""


@pytest.mark.parametrize("tune", ["M=2,T=256,B=2", "M=3,T=128,B=3", "M=4,T=128,B=2"])
def test_staged_eval_kernel_compiles(tune):
    env = dict(os.environ, RAL_EVAL_TUNE=tune)
    out = subprocess.run([sys.executable, "-c", SCRIPT % (PKG, ROOT)], env=env, capture_output=True, text=True,
                         check=True).stdout
    res = json.loads(out.strip().splitlines()[-1])
    # five input columns and their five masks, one bulk copy each per stage fill
    assert res["bulk"] == 10 and res["wait"]
    assert "error" not in res["log"].lower()
    assert "spill" not in res["log"] or "0 bytes spill stores" in res["log"]
