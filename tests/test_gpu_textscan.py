"""Scan -> filter fusion over delimited text on the GPU: ral_text_scan_filter against the oracle's
scan (oracle/textscan.py) followed by its process_filter, bit for bit (data of valid rows, masks,
null counts, row order), over tables that exercise the field rules and a 2M-row lineitem-like one."""
import numpy as np
import pytest

import helpers as H
import oracle as O
import ralgpu as R
from oracle import textscan as T
from ralgpu import dtypes as D
from ralgpu import workloads as W

pytestmark = pytest.mark.gpu


def _check(text, dtypes, proj, fq, **kw):
    """Both ways in: text already on the device, and text in host memory streamed in pieces."""
    exp = T.scan_filter(text, dtypes, proj, fq, **kw)
    for k, e in enumerate(exp):
        O.update_null_count(e)
    for from_host in (False, True):
        got = R.text_scan_filter(text, dtypes, proj, fq, from_host=from_host, **kw)
        assert len(got) == len(exp)
        for k, (g, e) in enumerate(zip(got, exp)):
            H.assert_columns_equal(g, e, what=f"column {k} ({fq}, from host {from_host})")
    return got


FILTERS = [None,
           "LogicalFilter(condition=[>($2, 25)])",
           "LogicalFilter(condition=[AND(>=($6, 1995-01-01), <($6, 1996-01-01 00:00:00))])",
           "LogicalFilter(condition=[OR(IS NULL($3), <($4, 0.03))])",
           "LogicalFilter(condition=[AND(>($5, 0.02), <>(MOD($1, 3), 0), IS NOT NULL($7))])",
           "LogicalFilter(condition=[<(*($3, -(1, $4)), 100.5)])"]


@pytest.mark.parametrize("fq", FILTERS)
def test_varied_table_every_column(fq):
    text = W.text_table_varied(3000, seed=21)
    _check(text, W.TEXT_DTYPES, list(range(8)), fq, skip_rows=1)


@pytest.mark.parametrize("piece", ["1", "100", "4097", "65536"])
def test_host_text_in_small_pieces(monkeypatch, piece):
    """Host text cut into pieces of one line up to many: each piece's kept rows are appended at a
    row that is not a multiple of 32 (the mask word shared with the piece before)."""
    monkeypatch.setenv("RAL_SCAN_PIECE_BYTES", piece)
    text = W.text_table_varied(3000, seed=33)
    _check(text, W.TEXT_DTYPES, list(range(8)), FILTERS[4], skip_rows=1)
    _check(text, W.TEXT_DTYPES, [6, 0, 3], None, skip_rows=5)


def test_projection_order_and_repeats():
    text = W.text_table_varied(2000, seed=5)
    _check(text, W.TEXT_DTYPES, [6, 0, 6, 3], "LogicalFilter(condition=[>($1, 0)])", skip_rows=1)


def test_lineitem_q6_2M_rows():
    text, _ = W.text_table(2_000_003, seed=9, values=True)
    got = _check(text, W.TEXT_DTYPES, W.TEXT_PROJECTIONS, W.TEXT_FILTER)
    assert 0.005 < got[0].size / 2_000_003 < 0.05


def test_reference_csv_test_file_layout():
    """The reference's CSV test table (tests/io-test/parse_csv.cu): 10 rows of 5 '|'-separated int32
    columns, value = row * (column * 3), a final newline; every value read back."""
    rows = ["|".join(str(r * (c * 3)) for c in range(5)) for r in range(10)]
    text = ("\n".join(rows) + "\n").encode()
    got = R.text_scan_filter(text, [D.GDF_INT32] * 5, [0, 1, 2, 3, 4])
    for c in range(5):
        assert got[c].to_numpy().tolist() == [r * (c * 3) for r in range(10)]
        assert got[c].null_count == 0


@pytest.mark.parametrize("text", [b"", b"\n\n\n", b"5|6", b"5|6\n", b"\r\n5|6\r\n\r\n7|x\n", b"a|b\n1|2\n"])
def test_small_inputs(text):
    _check(text, [D.GDF_INT32, D.GDF_INT64], [0, 1], None)
    _check(text, [D.GDF_INT32, D.GDF_INT64], [1], "LogicalFilter(condition=[>($0, 5)])")


def test_other_delimiter_and_terminator():
    text = b"1,2.5;3,x;;5,1e3;"
    _check(text, [D.GDF_INT32, D.GDF_FLOAT64], [0, 1], None, delimiter=b",", line_terminator=b";")


def test_refused_decimal_fails_the_call():
    text = b"1|2.5\n2|0.12345678901234567891\n3|4\n"
    with pytest.raises(T.ScanRefused):
        T.scan_filter(text, [D.GDF_INT32, D.GDF_FLOAT64], [0, 1], None)
    for from_host in (False, True):
        with pytest.raises(R.RalError):
            R.text_scan_filter(text, [D.GDF_INT32, D.GDF_FLOAT64], [0, 1], from_host=from_host)
    # a refused field in a row the filter drops, in a column the condition does not read: no error
    _check(text, [D.GDF_INT32, D.GDF_FLOAT64], [0, 1], "LogicalFilter(condition=[<>($0, 2)])")


def test_capacity_below_the_kept_rows_fails():
    text = b"1\n2\n3\n4\n"
    for from_host in (False, True):
        with pytest.raises(R.RalError):
            R.text_scan_filter(text, [D.GDF_INT32], [0], capacity=2, from_host=from_host)
    assert R.text_scan_rows(text) == 4 and R.text_scan_rows(text, skip_rows=3) == 1
