"""The integer-pipe IEEE-754 double operations (csrc/softfp.cuh), built for the host and checked
bit for bit against the host's own IEEE operations on edge cases and random inputs."""
import os
import shutil
import subprocess

import pytest

from conftest import PKG, ROOT


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("softfp") / "softfp_check")
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(PKG, "csrc"),
                           os.path.join(ROOT, "tests", "softfp", "softfp_check.cpp"), "-o", out])
    return out


def test_every_operation_matches_ieee(checker):
    res = subprocess.run([checker, "2000000"], capture_output=True, text=True, check=True).stdout
    rows = {}
    for line in res.strip().splitlines():
        name, n, bad, *first = line.split(" ", 3)
        rows[name] = (int(n), int(bad), first[0] if first else "")
    for name in ("sincos", "div64_32", "div64", "div", "floor", "ceil", "fabs", "compare", "i2d", "d2i", "f2d", "d2f", "is_zero"):
        n, bad, first = rows[name]
        assert n >= 1_000_000 and bad == 0, f"{name}: {bad} of {n} differ, first {first}"
