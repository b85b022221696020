"""CPU ORACLE of the delimited-text table scan (test infrastructure only).

Restates the scan the reference runs for a BindableTableScan over a CSV table
(src/CalciteInterpreter.cpp:745-767: the `projects=[...]` list picks the file
columns; src/io/data_parser/CSVParser.cpp:24-44,176-233: cudf's CSV reader with
'|' as the default delimiter, no header row, blank lines skipped), followed by
the LogicalFilter over the scanned frame (src/CalciteInterpreter.cpp:509-573,
restated by oracle.process_filter).  The CSV reader itself lives in cudf
(pinned by the reference to the 0.7/0.8 releases), which is not part of the
reference tree; the field rules below are the ones this project specifies for
numeric and date columns, and the library's scan kernel follows the same rules
(csrc/textscan.cuh):

* rows end at the line terminator (a '\\r' before it is dropped); the first
  `skip_rows` lines are skipped; empty lines are skipped;
* fields are split at the delimiter; spaces around a field are ignored; a
  missing, empty or unreadable field is null;
* integers: optional sign and digits, modulo 2**64, narrowed to the width;
* floating point: optional sign, digits with an optional point, optional
  exponent of at most five digits; rounded to the nearest double (then to float
  for FLOAT32).  Values whose significand has more than 19 significant digits,
  does not fit in 53 bits, or needs a power of ten beyond 1e22 are refused;
* dates: YYYY-MM-DD (DATE32 days, DATE64 milliseconds; DATE64 also accepts
  ' HH:MM:SS' or 'THH:MM:SS').
"""
from __future__ import annotations

import datetime
import re
from typing import List, Optional, Sequence

import numpy as np

from . import frontend as fe

NULL, OK, REFUSED = 0, 1, 2

_INT_RE = re.compile(rb"[+-]?[0-9]+\Z")
_EPOCH = datetime.date(1970, 1, 1)


class ScanRefused(ValueError):
    """A field value the scan refuses to round (outside the exact decimal range)."""


def parse_int(field: bytes):
    f = field.strip(b" ")
    if not _INT_RE.match(f):
        return NULL, 0
    v = int(f) % (1 << 64)
    return OK, v - (1 << 64) if v >= (1 << 63) else v


def parse_double(field: bytes):
    """(status, value) with the scan's rules: the significant digits and decimal exponent are
    found the way the kernel finds them, and an exact value is rounded by Python's float()."""
    f = field.strip(b" ")
    if not f:
        return NULL, 0.0
    i, n = 0, len(f)
    neg = False
    if f[i:i + 1] in (b"+", b"-"):
        neg = f[i:i + 1] == b"-"
        i += 1
    m, sig, e10, digits, dot = 0, 0, 0, 0, False
    while i < n:
        c = f[i:i + 1]
        if c == b".":
            if dot:
                return NULL, 0.0
            dot = True
            i += 1
            continue
        if not c.isdigit():
            break
        digits += 1
        d = c[0] - 48
        if m == 0 and d == 0:
            if dot:
                e10 -= 1
            i += 1
            continue
        if sig == 19:
            if d != 0:
                return REFUSED, 0.0
            if not dot:
                e10 += 1
            i += 1
            continue
        m = m * 10 + d
        sig += 1
        if dot:
            e10 -= 1
        i += 1
    if digits == 0:
        return NULL, 0.0
    if i < n:
        if f[i:i + 1] not in (b"e", b"E"):
            return NULL, 0.0
        i += 1
        eneg = False
        if i < n and f[i:i + 1] in (b"+", b"-"):
            eneg = f[i:i + 1] == b"-"
            i += 1
        if i >= n:
            return NULL, 0.0
        x, nd = 0, 0
        while i < n:
            c = f[i:i + 1]
            if not c.isdigit():
                return NULL, 0.0
            nd += 1
            if nd > 5:
                return REFUSED, 0.0
            x = x * 10 + (c[0] - 48)
            i += 1
        e10 += -x if eneg else x
    if m == 0:
        v = 0.0
    else:
        two53 = 1 << 53
        while e10 > 22 and m <= two53 // 10:
            m *= 10
            e10 -= 1
        if m > two53 or e10 > 22 or e10 < -22:
            return REFUSED, 0.0
        # the decimal m * 10^e10 rounded once to the nearest double
        v = float(m * 10 ** e10) if e10 >= 0 else m / 10 ** (-e10)
    return OK, -v if neg else v


def parse_date(field: bytes, with_time: bool):
    f = field.strip(b" ")
    n = len(f)
    if n < 10 or f[4:5] != b"-" or f[7:8] != b"-":
        return NULL, 0
    y, mo, d = f[0:4], f[5:7], f[8:10]
    if not (y.isdigit() and mo.isdigit() and d.isdigit()):
        return NULL, 0
    try:
        days = (datetime.date(int(y), int(mo), int(d)) - _EPOCH).days
    except ValueError:
        return NULL, 0
    if not with_time:
        return (OK, days) if n == 10 else (NULL, 0)
    secs = 0
    if n != 10:
        if n != 19 or f[10:11] not in (b" ", b"T") or f[13:14] != b":" or f[16:17] != b":":
            return NULL, 0
        h, mi, s = f[11:13], f[14:16], f[17:19]
        if not (h.isdigit() and mi.isdigit() and s.isdigit()):
            return NULL, 0
        h, mi, s = int(h), int(mi), int(s)
        if h > 23 or mi > 59 or s > 59:
            return NULL, 0
        secs = h * 3600 + mi * 60 + s
    return OK, (days * 86400 + secs) * 1000


def _narrow(v: int, dtype: int) -> int:
    bits = {fe.GDF_INT8: 8, fe.GDF_INT16: 16, fe.GDF_INT32: 32, fe.GDF_INT64: 64}[dtype]
    v &= (1 << bits) - 1
    return v - (1 << bits) if v >= 1 << (bits - 1) else v


def parse_field(field: bytes, dtype: int):
    if dtype in (fe.GDF_INT8, fe.GDF_INT16, fe.GDF_INT32, fe.GDF_INT64):
        st, v = parse_int(field)
        return st, _narrow(v, dtype) if st == OK else 0
    if dtype in (fe.GDF_FLOAT32, fe.GDF_FLOAT64):
        return parse_double(field)
    if dtype == fe.GDF_DATE32:
        return parse_date(field, False)
    if dtype == fe.GDF_DATE64:
        return parse_date(field, True)
    raise ValueError(f"dtype {dtype} is not scanned")


def split_rows(data: bytes, line_terminator: bytes = b"\n", skip_rows: int = 0) -> List[bytes]:
    lines = data.split(line_terminator)
    if data.endswith(line_terminator):
        lines = lines[:-1]                    # the terminator ends the last line
    rows = []
    for k, ln in enumerate(lines):
        if k < skip_rows:
            continue
        if ln.endswith(b"\r"):
            ln = ln[:-1]
        if ln:
            rows.append(ln)
    return rows


def _scan_status(data, file_dtypes, projections, delimiter, line_terminator, skip_rows):
    """The scanned frame (refused fields read as null, as the kernel reads them) and each field's
    status (NULL / OK / REFUSED), per projected column."""
    from . import make_column, NP_DTYPE
    rows = split_rows(data, line_terminator, skip_rows)
    cols, status = [], []
    for c in projections:
        dt = file_dtypes[c]
        vals = np.zeros(len(rows), dtype=NP_DTYPE[dt])
        st_col = np.zeros(len(rows), dtype=np.int8)
        for r, row in enumerate(rows):
            fields = row.split(delimiter)
            if c >= len(fields):
                continue
            st, v = parse_field(fields[c], dt)
            st_col[r] = st
            if st == OK:
                vals[r] = v
        cols.append(make_column(vals, dt, st_col == OK))
        status.append(st_col)
    return cols, status


def scan(data: bytes, file_dtypes: Sequence[int], projections: Sequence[int], delimiter: bytes = b"|",
         line_terminator: bytes = b"\n", skip_rows: int = 0):
    """The scanned frame: one OColumn per projected file column (every column carries a mask)."""
    cols, status = _scan_status(data, file_dtypes, projections, delimiter, line_terminator, skip_rows)
    for k, st in enumerate(status):
        bad = np.nonzero(st == REFUSED)[0]
        if bad.size:
            raise ScanRefused(f"row {bad[0]} of scanned column {k}")
    return cols


def scan_filter(data: bytes, file_dtypes, projections, filter_query_part: Optional[str], delimiter: bytes = b"|",
                line_terminator: bytes = b"\n", skip_rows: int = 0):
    """BindableTableScan followed by its LogicalFilter (None: the scan alone).  A refused field
    fails the scan where the kernel parses it: in a column the condition reads (every row), or in
    any projected column of a kept row."""
    from . import process_filter, filter_indices, materialize_column
    cols, status = _scan_status(data, file_dtypes, projections, delimiter, line_terminator, skip_rows)
    n = cols[0].size if cols else 0
    if filter_query_part is None:
        keep = np.arange(n, dtype=np.int32)
    else:
        cond = fe.get_named_expression(filter_query_part, "condition")
        for k in {int(m) for m in re.findall(r"\$(\d+)", cond)}:
            if k < len(status) and (status[k] == REFUSED).any():
                raise ScanRefused(f"scanned column {k}, read by the condition")
        keep = filter_indices(cols, filter_query_part)
    for k, st in enumerate(status):
        if (st[keep] == REFUSED).any():
            raise ScanRefused(f"scanned column {k} of a kept row")
    if filter_query_part is None:
        return cols
    return process_filter(cols, filter_query_part)
