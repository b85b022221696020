"""Parquet metadata on the host: the minimal writer of ralgpu.workloads reads back in pyarrow (where
it is installed), the footer reader gives the fixtures' schemas, and unsupported files are refused
before any device work."""
import ctypes
import io
import os

import numpy as np
import pytest

import ralgpu as R
from conftest import ROOT
from ralgpu import dtypes as D
from ralgpu import workloads as W

GOLDEN = os.path.join(ROOT, "tests", "golden")


def _writer_table(n, seed):
    rng = np.random.default_rng(seed)
    va = rng.random(n) >= 0.1
    va[100:400] = True          # a long run of present levels (an RLE run)
    va[500:700] = False         # a long run of nulls
    cols = [("a", D.GDF_INT32, rng.integers(-99, 99, n).astype(np.int32), va),
            ("b", D.GDF_FLOAT64, rng.standard_normal(n), None),
            ("c", D.GDF_DATE32, rng.integers(0, 20000, n).astype(np.int32), rng.random(n) >= 0.5),
            ("d", D.GDF_DATE64, rng.integers(0, 10**12, n).astype(np.int64), None),
            ("e", D.GDF_FLOAT32, rng.standard_normal(n).astype(np.float32), rng.random(n) >= 0.02),
            ("f", D.GDF_INT64, rng.integers(-(1 << 60), 1 << 60, n).astype(np.int64), None)]
    return cols


@pytest.mark.parametrize("snappy,dictionary", [(False, False), (True, False), (False, True), (True, True)])
def test_writer_output_reads_back_in_pyarrow(snappy, dictionary):
    pq = pytest.importorskip("pyarrow.parquet")
    cols = _writer_table(20_000, 1)
    if dictionary:  # few distinct values in some columns, too many (PLAIN pages) in others
        cols[0] = (cols[0][0], cols[0][1], (cols[0][2] % 7).astype(np.int32), cols[0][3])
        cols[3] = (cols[3][0], cols[3][1], (cols[3][2] % 1000).astype(np.int64), cols[3][3])
    b = W.parquet_bytes(cols, row_group_rows=7000, page_rows=3000, snappy=snappy, dictionary=dictionary,
                        dictionary_max=1000)
    if dictionary:
        md = pq.ParquetFile(io.BytesIO(b)).metadata.row_group(0)
        assert [md.column(k).has_dictionary_page for k in range(6)] == [True, False, False, True, False, False]
    t = pq.read_table(io.BytesIO(b))
    for name, dt, v, m in cols:
        c = t.column(name)
        got_valid = np.asarray(c.is_valid())
        assert np.array_equal(got_valid, np.ones(len(v), bool) if m is None else m), name
        import pyarrow as pa
        raw = c.cast(pa.int64() if dt in (D.GDF_DATE64,) else (pa.int32() if dt == D.GDF_DATE32 else c.type)).fill_null(0)
        arr = raw.to_numpy()
        keep = got_valid
        assert np.array_equal(arr[keep].astype(v.dtype).view(np.uint8), v[keep].view(np.uint8)), name


def test_schema_of_the_fixtures():
    b = open(os.path.join(GOLDEN, "parquet_plain.parquet"), "rb").read()
    rows, dts = R.parquet_schema(b)
    assert rows == 3000
    # g is a string leaf: no scanned dtype
    assert dts == [D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64, D.GDF_DATE32, D.GDF_DATE64, D.GDF_invalid]
    b = W.parquet_bytes(_writer_table(5000, 2), row_group_rows=2000, page_rows=700)
    rows, dts = R.parquet_schema(b)
    assert rows == 5000 and dts == [D.GDF_INT32, D.GDF_FLOAT64, D.GDF_DATE32, D.GDF_DATE64, D.GDF_FLOAT32, D.GDF_INT64]


@pytest.mark.parametrize("name,leaf,reason", [("parquet_gzip", 0, "Snappy-compressed"),
                                              ("parquet_plain", 6, "columns are scanned"),
                                              ("parquet_delta", 1, "page encoding")])
def test_unsupported_files_are_refused_before_device_work(name, leaf, reason):
    b = open(os.path.join(GOLDEN, name + ".parquet"), "rb").read()
    rows, dts = R.parquet_schema(b)
    L = R.lib()
    # out columns with placeholder pointers: the refusal comes before anything is dereferenced
    outs = (R.capi.GdfColumn * 1)()
    outs[0].data = ctypes.c_void_p(256)
    outs[0].valid = ctypes.c_void_p(256)
    outs[0].size = rows
    outs[0].dtype = dts[leaf]
    ptrs = (ctypes.c_void_p * 1)(ctypes.addressof(outs[0]))
    pr = (ctypes.c_int32 * 1)(leaf)
    n = ctypes.c_int32(0)
    buf = ctypes.create_string_buffer(b, len(b))
    rc = L.ral_parquet_scan_filter(buf, len(b), pr, 1, None, ctypes.cast(ptrs, ctypes.c_void_p), ctypes.byref(n))
    assert rc != 0 and reason in L.ral_last_error().decode()


def test_not_parquet_and_truncated():
    with pytest.raises(R.RalError):
        R.parquet_schema(b"PAR1 not a parquet file")
    b = open(os.path.join(GOLDEN, "parquet_plain.parquet"), "rb").read()
    with pytest.raises(R.RalError):
        R.parquet_schema(b[:-20] + b[-8:])


FIXTURES = ["parquet_plain", "parquet_snappy", "parquet_dictionary", "parquet_dict_fallback", "parquet_v2",
            "parquet_v2_snappy_dict", "parquet_defaults"]
FIXTURE_DTYPES = [D.GDF_INT32, D.GDF_INT64, D.GDF_FLOAT32, D.GDF_FLOAT64, D.GDF_DATE32, D.GDF_DATE64]


def _same_column(got, values, valid, what):
    n = len(values)
    assert got.size == n, what
    gv = got.valid_bools()
    assert np.array_equal(gv, valid), what
    a = got.data[valid].view(np.uint8)
    b = np.ascontiguousarray(np.asarray(values)[valid]).astype(got.data.dtype).view(np.uint8)
    assert np.array_equal(a, b), what


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_reads_the_pyarrow_fixtures(name):
    """The oracle's Parquet reader against the values pyarrow wrote (pins the oracle)."""
    from oracle import parquet as OP
    b = open(os.path.join(GOLDEN, name + ".parquet"), "rb").read()
    v = np.load(os.path.join(GOLDEN, name + ".npz"))
    n = len(v["b"])
    ones = np.ones(n, bool)
    cols = OP.scan(b, list(range(6)))
    for k, (key, m) in enumerate([("a", v["a_valid"]), ("b", ones), ("c", v["c_valid"]), ("d", ones),
                                  ("e", v["e_valid"]), ("f", ones)]):
        assert cols[k].dtype == FIXTURE_DTYPES[k]
        _same_column(cols[k], v[key], m, f"{name} {key}")
    with pytest.raises(OP.Unsupported):
        OP.scan(b, [6])  # the string leaf


@pytest.mark.parametrize("snappy,dictionary", [(False, False), (True, False), (False, True), (True, True)])
def test_oracle_reads_the_writer_files(snappy, dictionary):
    from oracle import parquet as OP
    cols = _writer_table(5000, 11)
    b = W.parquet_bytes(cols, row_group_rows=2000, page_rows=700, snappy=snappy, dictionary=dictionary,
                        dictionary_max=3000)
    got = OP.scan(b, list(range(6)))
    for k, (name, dt, v, m) in enumerate(cols):
        _same_column(got[k], v, np.ones(len(v), bool) if m is None else m, f"{name}")


def test_oracle_hybrid_runs():
    """The RLE / bit-packed hybrid: RLE runs, bit-packed runs padded to whole groups, width 0."""
    from oracle import parquet as OP
    # RLE: 5 x value 3 (width 2: one byte), then bit-packed: 1 group of 8 values 0..7 at width 3
    buf = bytes([5 << 1, 3]) + bytes([(1 << 1) | 1]) + bytes([0b10001000, 0b11000110, 0b11111010])
    got = OP.hybrid(buf, 0, len(buf), 3, 13)
    assert got.tolist() == [3] * 5 + list(range(8))
    # only the first 6 of a padded group are asked for
    assert OP.hybrid(buf, 2, len(buf), 3, 6).tolist() == list(range(6))
    # width 0: every value 0
    assert OP.hybrid(bytes([(2 << 1) | 1]), 0, 1, 0, 16).tolist() == [0] * 16
    with pytest.raises(OP.Unsupported):
        OP.hybrid(bytes([4 << 1, 1]), 0, 2, 1, 5)  # runs end before the values do


def test_oracle_snappy_back_references():
    """Raw Snappy: a literal, then an overlapping copy (offset 1 repeats one byte)."""
    from oracle import parquet as OP
    # length 7, literal "ab" (tag (2-1) << 2), copy of 5 bytes at offset 1 (1-byte offset form:
    # len 4 + ((tag >> 2) & 7), offset (tag >> 5) << 8 | next byte)
    stream = bytes([7, (2 - 1) << 2]) + b"ab" + bytes([((5 - 4) << 2) | 1, 1])
    assert OP.snappy_decompress(stream) == b"abbbbbb"
    with pytest.raises(OP.Unsupported):
        OP.snappy_decompress(bytes([8, (2 - 1) << 2]) + b"ab" + bytes([((5 - 4) << 2) | 1, 1]))
