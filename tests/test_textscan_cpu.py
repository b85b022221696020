"""The text-scan field parsers (csrc/textscan.cuh), built for the host and compared value for value
with the oracle's restatement (oracle/textscan.py) on edge cases and random fields."""
import os
import random
import shutil
import struct
import subprocess

import pytest

from conftest import PKG, ROOT
from oracle import textscan as T
from oracle import frontend as fe


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("textscan") / "textscan_check")
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(PKG, "csrc"),
                           os.path.join(ROOT, "tests", "textscan", "textscan_check.cpp"), "-o", out])
    return out


def _run(checker, cases):
    inp = "".join(f"{k} {f.hex()}\n" for k, f in cases)
    out = subprocess.run([checker], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    res = []
    for line in out[:len(cases)]:
        st, v = line.split()
        res.append((int(st), int(v)))
    return res


def _expect(kind, field):
    if kind == "i":
        st, v = T.parse_int(field)
        return st, v if st == T.OK else 0
    if kind == "f":
        st, v = T.parse_double(field)
        return st, struct.unpack("<q", struct.pack("<d", v))[0] if st == T.OK else 0
    st, v = T.parse_date(field, kind == "t")
    return st, v if st == T.OK else 0


EDGE = [b"", b" ", b"0", b"-0", b"+0", b"00012", b" 42 ", b"-", b"+", b"1-", b"12a", b"9223372036854775807",
        b"9223372036854775808", b"-9223372036854775808", b"18446744073709551616", b"99999999999999999999999",
        b"1.5", b".5", b"5.", b".", b"1e5", b"1E-5", b"1e", b"1e+", b"-1.25e-3", b"0.000", b"0e999999",
        b"9007199254740993", b"9007199254740992", b"1e22", b"1e23", b"123e21", b"1e-22", b"1e-23",
        b"0.1", b"0.30000000000000004", b"1234567890123456789", b"12345678901234567890", b"1.0000000000000000000",
        b"1e100000", b"inf", b"nan", b"1.2.3", b"--1", b"1 2",
        b"1970-01-01", b"2000-02-29", b"1900-02-29", b"2019-13-01", b"2019-12-32", b"2019-1-01", b"0000-01-01",
        b"9999-12-31", b"2019-06-15 12:30:45", b"2019-06-15T23:59:59", b"2019-06-15 24:00:00", b"2019-06-15 12:30",
        b" 1995-03-15 "]


def test_edge_fields_match_the_oracle(checker):
    cases = [(k, f) for f in EDGE for k in "ifdt"]
    got = _run(checker, cases)
    for (k, f), g in zip(cases, got):
        assert g == _expect(k, f), (k, f, g, _expect(k, f))


def _rand_decimal(rng):
    digits = rng.randint(1, 21)
    s = "".join(rng.choice("0123456789") for _ in range(digits))
    if rng.random() < 0.7:
        p = rng.randint(0, len(s))
        s = s[:p] + "." + s[p:]
    if rng.random() < 0.4:
        s += rng.choice("eE") + rng.choice(["", "+", "-"]) + str(rng.randint(0, 40))
    if rng.random() < 0.3:
        s = rng.choice("+-") + s
    return s.encode()


def test_random_fields_match_the_oracle(checker):
    rng = random.Random(7)
    cases = []
    for _ in range(60000):
        cases.append(("f", _rand_decimal(rng)))
        cases.append(("i", str(rng.randint(-(1 << 70), 1 << 70)).encode()))
        y, m, d = rng.randint(1, 9999), rng.randint(0, 13), rng.randint(0, 32)
        cases.append(("d" if rng.random() < 0.5 else "t", f"{y:04d}-{m:02d}-{d:02d}".encode()))
    got = _run(checker, cases)
    bad = [(k, f, g, _expect(k, f)) for (k, f), g in zip(cases, got) if g != _expect(k, f)]
    assert not bad, bad[:5]
    ok = sum(1 for (k, f), g in zip(cases, got) if k == "f" and g[0] == T.OK)
    assert ok > 20000


def test_exact_decimals_are_correctly_rounded(checker):
    """Fields in the exact range give the double nearest to the decimal (Python's float())."""
    rng = random.Random(11)
    cases = []
    for _ in range(40000):
        m = rng.randint(0, (1 << 53))
        e = rng.randint(-22, 22)
        cases.append(("f", f"{m}e{e}".encode()))
        cases.append(("f", f"{rng.randint(0, 10**9)}.{rng.randint(0, 99):02d}".encode()))
    got = _run(checker, cases)
    for (k, f), (st, bits) in zip(cases, got):
        assert st == T.OK, f
        assert bits == struct.unpack("<q", struct.pack("<d", float(f)))[0], f


@pytest.mark.parametrize("host", [False, True])
def test_scan_arguments_are_checked_before_device_work(host):
    """Both entry points refuse bad arguments on the host (no device is touched): the delimiter equal
    to the line terminator, a projection outside the file, an unscannable column type."""
    import ctypes
    import ralgpu as R
    L = R.lib()
    fn = L.ral_text_scan_filter_host if host else L.ral_text_scan_filter
    text = ctypes.create_string_buffer(b"1|2\n3|4\n")
    fd = (ctypes.c_int32 * 2)(fe.GDF_INT32, fe.GDF_INT32)
    outs = (R.capi.GdfColumn * 1)()
    outs[0].data = ctypes.c_void_p(256)
    outs[0].valid = ctypes.c_void_p(256)
    outs[0].size = 2
    outs[0].dtype = fe.GDF_INT32
    ptrs = (ctypes.c_void_p * 1)(ctypes.addressof(outs[0]))
    n = ctypes.c_int32(0)
    for delim, term, proj, why in [(b"|", b"|", 0, "same byte"), (b"|", b"\n", 5, "out of range")]:
        pr = (ctypes.c_int32 * 1)(proj)
        rc = fn(text, 8, delim, term, 0, fd, 2, pr, 1, None, ctypes.cast(ptrs, ctypes.c_void_p), ctypes.byref(n))
        assert rc != 0 and why in L.ral_last_error().decode()
    fd_bad = (ctypes.c_int32 * 2)(fe.GDF_INT32, fe.GDF_STRING_CATEGORY)
    pr = (ctypes.c_int32 * 1)(1)
    rc = fn(text, 8, b"|", b"\n", 0, fd_bad, 2, pr, 1, None, ctypes.cast(ptrs, ctypes.c_void_p), ctypes.byref(n))
    assert rc != 0 and "floating-point and date" in L.ral_last_error().decode()
