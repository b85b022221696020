"""Scan -> filter over Parquet on the GPU: ral_parquet_scan_filter against the values each file
holds (pyarrow's fixtures with their .npz, and files of ralgpu.workloads.parquet_bytes) and the
oracle's process_filter over them, bit for bit; required and optional leaves, many pages and row
groups, RLE and bit-packed definition levels, v1 and v2 pages, PLAIN values and dictionary indices
(with pyarrow's fallback to PLAIN pages), uncompressed and Snappy chunks, pyarrow's defaults."""
import os

import numpy as np
import pytest

import helpers as H
import oracle as O
import ralgpu as R
from conftest import ROOT
from ralgpu import dtypes as D
from ralgpu import workloads as W
from test_parquet_cpu import _writer_table

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(ROOT, "tests", "golden")

FILTERS = [None,
           "LogicalFilter(condition=[>($0, 0)])",
           "LogicalFilter(condition=[OR(IS NULL($2), <($3, 0))])",
           "LogicalFilter(condition=[AND(>=($4, 1995-01-01), <($1, 0))])",
           "LogicalFilter(condition=[<(*($3, 2), $2)])"]


def _check(file_bytes, frame, proj, fq):
    """Both ways in: pages copied from pageable memory, and read in place from page-locked memory;
    against the values the file was written from and against the oracle's own read of the file."""
    from oracle import parquet as OP
    exp_frame = [frame[c] for c in proj]
    exp = exp_frame if fq is None else O.process_filter(exp_frame, fq)
    ora = OP.scan_filter(file_bytes, proj, fq)
    assert len(ora) == len(exp)
    for k, (a, e) in enumerate(zip(ora, exp)):
        av, ev = a.valid_bools(), e.valid_bools()
        assert np.array_equal(av, ev), f"oracle column {k} ({fq}): validity"
        assert np.array_equal(a.data[av].view(np.uint8), e.data[ev].view(np.uint8)), f"oracle column {k} ({fq}): data"
    for page_locked in (False, True):
        got = R.parquet_scan_filter(file_bytes, proj, fq, page_locked=page_locked)
        assert len(got) == len(exp)
        for k, (g, e) in enumerate(zip(got, exp)):
            O.update_null_count(e)
            H.assert_columns_equal(g, e, what=f"column {k} ({fq}, page-locked {page_locked})")


PYARROW_FILES = ["parquet_plain", "parquet_snappy", "parquet_dictionary", "parquet_dict_fallback", "parquet_v2",
                 "parquet_v2_snappy_dict", "parquet_defaults"]


@pytest.mark.parametrize("name", PYARROW_FILES)
@pytest.mark.parametrize("fq", FILTERS)
def test_pyarrow_fixture(name, fq):
    b = open(os.path.join(GOLDEN, name + ".parquet"), "rb").read()
    v = np.load(os.path.join(GOLDEN, name + ".npz"))
    n = len(v["b"])
    ones = np.ones(n, bool)
    frame = [O.make_column(v["a"], D.GDF_INT32, v["a_valid"]), O.make_column(v["b"], D.GDF_INT64, ones),
             O.make_column(v["c"], D.GDF_FLOAT32, v["c_valid"]), O.make_column(v["d"], D.GDF_FLOAT64, ones),
             O.make_column(v["e"], D.GDF_DATE32, v["e_valid"]), O.make_column(v["f"], D.GDF_DATE64, ones)]
    _check(b, frame, [0, 1, 2, 3, 4, 5], fq)


def _frame_of(cols):
    return [O.make_column(v, dt, np.ones(len(v), bool) if m is None else m) for _, dt, v, m in cols]


@pytest.mark.parametrize("rows,rg,page", [(1, 1, 1), (33, 10, 7), (5000, 2000, 700), (1_000_003, 300_000, 65_536),
                                          (600_000, 600_000, 300_000)])
def test_writer_files(rows, rg, page):
    # the last case: pages whose levels exceed the 32 KiB staged in shared memory and hold more
    # than the 1024 runs of one table batch
    cols = _writer_table(rows, rows)
    b = W.parquet_bytes(cols, row_group_rows=rg, page_rows=page)
    frame = _frame_of(cols)
    _check(b, frame, [0, 1, 2, 3, 4, 5], None)
    # projections reorder the scanned frame: $0 = a, $1 = f, $2 = c, $3 = b, $4 = d
    _check(b, frame, [0, 5, 2, 1, 3], "LogicalFilter(condition=[OR(IS NULL($2), <($3, 0))])")


def test_unsupported_files_fail_cleanly():
    for page_locked in (False, True):
        with pytest.raises(R.RalError):  # a GZIP-compressed file
            R.parquet_scan_filter(open(os.path.join(GOLDEN, "parquet_gzip.parquet"), "rb").read(), [0, 1],
                                  page_locked=page_locked)
        with pytest.raises(R.RalError):  # a string leaf
            R.parquet_scan_filter(open(os.path.join(GOLDEN, "parquet_plain.parquet"), "rb").read(), [6],
                                  page_locked=page_locked)
    # the context stays usable
    good = W.parquet_bytes(_writer_table(100, 5))
    assert R.parquet_scan_filter(good, [0])[0].size == 100


@pytest.mark.parametrize("rows,rg,page", [(33, 10, 7), (5000, 2000, 700), (300_001, 100_000, 65_536)])
def test_writer_files_snappy(rows, rg, page):
    """The project writer's Snappy chunks (literal-only streams, long literals with 2-byte lengths)."""
    cols = _writer_table(rows, rows + 1)
    b = W.parquet_bytes(cols, row_group_rows=rg, page_rows=page, snappy=True)
    frame = _frame_of(cols)
    _check(b, frame, [0, 1, 2, 3, 4, 5], None)
    _check(b, frame, [0, 5, 2, 1, 3], "LogicalFilter(condition=[OR(IS NULL($2), <($3, 0))])")


@pytest.mark.parametrize("rows,rg,page,snappy", [(33, 10, 7, False), (5000, 2000, 700, True),
                                                (300_001, 100_000, 65_536, False)])
def test_writer_files_dictionary(rows, rg, page, snappy):
    """The project writer's dictionary-encoded chunks: index bit widths 0 (one entry), 1, 10 and 16,
    optional and required leaves, chunks past the dictionary cap written as PLAIN pages."""
    cols = _writer_table(rows, rows + 2)
    cols[0] = (cols[0][0], cols[0][1], np.full(rows, 7, np.int32), cols[0][3])                 # one entry
    cols[2] = (cols[2][0], cols[2][1], (cols[2][2] % 2).astype(np.int32), cols[2][3])          # two
    cols[3] = (cols[3][0], cols[3][1], (cols[3][2] % 1000).astype(np.int64), cols[3][3])       # 1000
    cols[4] = (cols[4][0], cols[4][1], np.round(cols[4][2] * 8000).astype(np.float32), cols[4][3])
    b = W.parquet_bytes(cols, row_group_rows=rg, page_rows=page, snappy=snappy, dictionary=True,
                        dictionary_max=40_000)
    frame = _frame_of(cols)
    _check(b, frame, [0, 1, 2, 3, 4, 5], None)
    _check(b, frame, [0, 5, 2, 1, 3, 4], "LogicalFilter(condition=[OR(IS NULL($2), <($4, 500))])")


@pytest.mark.parametrize("delta", [-1, 1])
def test_corrupt_snappy_page_is_an_error(delta):
    """Snappy streams whose stated length differs from their page's: the call fails, nothing faults."""
    b = W.parquet_bytes(_writer_table(5000, 2), row_group_rows=2000, page_rows=700, snappy=True,
                        snappy_length_delta=delta)
    for page_locked in (False, True):
        with pytest.raises(R.RalError):
            R.parquet_scan_filter(b, [0, 1], page_locked=page_locked)
    good = W.parquet_bytes(_writer_table(100, 5))
    assert R.parquet_scan_filter(good, [0])[0].size == 100
