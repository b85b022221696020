"""The header-only C++ wrappers (include/ral/ral.hpp) compile, link against libralgpu.so and
behave like the reference API on the host side (emitter output, exceptions) without a GPU."""
import os
import subprocess

import pytest

import ralgpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <cstdio>
#include <stdexcept>
#include "ral/ral.hpp"

int main() {
    // add_expression_to_plan over a 4-column frame, as LogicalFilter.cpp:338-351 calls it
    std::vector<column_index_type> l, r, o, nii = {0, 1, 2, 3};
    std::vector<gdf_binary_operator> ops;
    std::vector<gdf_unary_operator> uops;
    std::vector<gdf_scalar> ls, rs;
    ral::add_expression_to_plan("AND(=(*($0, $0), 1), =($1, 2))", 0, 1, 4, l, r, o, ops, uops, ls, rs, nii);
    std::printf("ops=%zu", ops.size());
    for (size_t k = 0; k < ops.size(); k++) std::printf(" [%d %d %d %d %d]", l[k], r[k], o[k], (int)ops[k], (int)uops[k]);
    std::printf("\n");
    // an invalid call throws std::runtime_error like the reference's CheckCudaErrors
    try {
        std::vector<gdf_column*> none;
        std::vector<column_index_type> e;
        std::vector<gdf_binary_operator> eo;
        std::vector<gdf_unary_operator> eu;
        std::vector<gdf_scalar> es;
        ral::perform_operation(none, none, e, e, e, e, eo, eu, es, es, e);
        std::printf("no exception\n");
        return 1;
    } catch (const std::runtime_error& ex) {
        std::printf("threw: %s\n", ex.what());
    }
    return 0;
}
"""


def test_cpp_wrappers(tmp_path):
    lib = ralgpu.lib()._name
    src = tmp_path / "w.cpp"
    src.write_text(SRC)
    exe = tmp_path / "w"
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    f"-L{libdir}", "-lralgpu", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    lines = out.strip().splitlines()
    # same program as the oracle's restatement of the reference emitter
    from oracle import frontend as fe
    plan = fe.Plan()
    fe.add_expression_to_plan("AND(=(*($0, $0), 1), =($1, 2))", 0, 1, 4, plan, [0, 1, 2, 3])
    exp = " ".join(f"[{a} {b} {c} {d} {e}]" for a, b, c, d, e in
                   zip(plan.left, plan.right, plan.outputs, plan.operators, plan.unary_operators))
    assert lines[0] == f"ops={len(plan.left)} {exp}"
    assert lines[1].startswith("threw: ralgpu:")
