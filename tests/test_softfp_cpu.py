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
    for name in ("sincos", "divc", "div64_16", "div64_32", "div64", "div", "div_rcp", "floor", "ceil", "fabs", "compare", "i2d", "d2i", "f2d", "d2f", "is_zero"):
        n, bad, first = rows[name]
        assert n >= 1_000_000 and bad == 0, f"{name}: {bad} of {n} differ, first {first}"


def test_sincos_constants_are_the_stated_values():
    """2/pi * 2^192 and pi/2 * 2^127 (truncated) and 2^63 / n! (nearest) in softfp.cuh, recomputed."""
    import re
    from fractions import Fraction
    from math import factorial
    mpmath = pytest.importorskip("mpmath")
    src = open(os.path.join(PKG, "csrc", "softfp.cuh")).read()
    d = {k: int(v, 16) for k, v in re.findall(r"#define (RAL_SF_\w+) (0x[0-9a-f]+)ull", src)}
    mpmath.mp.dps = 100
    two_pi = int(mpmath.floor(2 / mpmath.pi * mpmath.mpf(2) ** 192))
    assert (d["RAL_SF_2PI_W2"] << 128) | (d["RAL_SF_2PI_W1"] << 64) | d["RAL_SF_2PI_W0"] == two_pi
    pi2 = int(mpmath.floor(mpmath.pi / 2 * mpmath.mpf(2) ** 127))
    assert (d["RAL_SF_PI2_HI"] << 64) | d["RAL_SF_PI2_LO"] == pi2

    def nearest(n):
        return round(Fraction(2 ** 63, factorial(n)))

    arrays = re.findall(r"const unsigned long long c\[\d+\] = \{([^}]*)\}", src)
    cos_c = [int(v, 16) for v in re.findall(r"0x[0-9a-f]+", arrays[0])]
    sin_c = [int(v, 16) for v in re.findall(r"0x[0-9a-f]+", arrays[1])]
    assert cos_c == [nearest(2 * n) for n in range(11)]
    assert sin_c == [nearest(2 * n + 1) for n in range(10)]
