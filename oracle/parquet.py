"""CPU ORACLE of the Parquet table scan (test infrastructure only).

Restates the scan the reference runs for a BindableTableScan over a Parquet table
(src/CalciteInterpreter.cpp:745-767: `projects=[...]` picks the leaves;
src/io/data_parser/ParquetParser.cpp:36-90 hands the file to cudf's Parquet reader,
pinned by the reference to the cudf 0.7/0.8 releases and not part of its tree), followed
by the LogicalFilter over the scanned frame (process_filter).  The reader here follows
the published Apache Parquet format (footer and page headers in Thrift's compact
protocol with parquet.thrift's field ids; PLAIN values; the RLE / bit-packed hybrid for
definition levels and dictionary indices; DATA_PAGE and DATA_PAGE_V2) and the raw Snappy
format (google/snappy format_description.txt), for the subset the library scans: flat
schemas of INT32 (DATE), INT64 (TIMESTAMP_MILLIS), FLOAT and DOUBLE leaves, uncompressed
or SNAPPY chunks.  It is pinned by pyarrow's files with the values each holds
(tests/golden/parquet_*.parquet and .npz; tests/test_parquet_cpu.py).
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from . import frontend as fe

_NP = {1: np.int32, 2: np.int64, 4: np.float32, 5: np.float64}   # physical type -> values


class Unsupported(ValueError):
    """A file or page outside the subset the scan reads."""


class _Thrift:
    """Thrift compact protocol: fields (id delta << 4 | type), zigzag varints, lists, structs."""

    def __init__(self, b: bytes, pos: int):
        self.b, self.p, self.last = b, pos, [0]

    def byte(self) -> int:
        v = self.b[self.p]
        self.p += 1
        return v

    def varint(self) -> int:
        v, shift = 0, 0
        while True:
            c = self.byte()
            v |= (c & 0x7F) << shift
            shift += 7
            if not c & 0x80:
                return v

    def zigzag(self) -> int:
        v = self.varint()
        return (v >> 1) ^ -(v & 1)

    def field(self):
        h = self.byte()
        if h == 0:
            return None
        t, d = h & 0x0F, h >> 4
        fid = self.last[-1] + d if d else self.zigzag()
        self.last[-1] = fid
        return fid, t

    def list_header(self):
        h = self.byte()
        n = h >> 4
        return h & 0x0F, (self.varint() if n == 15 else n)

    def binary(self) -> bytes:
        n = self.varint()
        v = self.b[self.p:self.p + n]
        self.p += n
        return v

    def struct(self, on_field):
        self.last.append(0)
        while True:
            f = self.field()
            if f is None:
                break
            if not on_field(*f):
                self.skip(f[1])
        self.last.pop()

    def skip(self, t: int):
        if t in (1, 2):
            return
        if t == 3:
            self.byte()
        elif t in (4, 5, 6):
            self.varint()
        elif t == 7:
            self.p += 8
        elif t == 8:
            self.binary()
        elif t in (9, 10):
            et, n = self.list_header()
            for _ in range(n):
                self.skip(et)
        elif t == 11:
            n = self.varint()
            if n:
                kv = self.byte()
                for _ in range(n):
                    self.skip(kv >> 4)
                    self.skip(kv & 0x0F)
        elif t == 12:
            self.struct(lambda i, tt: False)
        else:
            raise Unsupported(f"thrift type {t}")


def read_footer(b: bytes) -> dict:
    """num_rows, leaves [(name, physical type, repetition, converted type)], row groups with their
    columns' (codec, num_values, data_page_offset, dictionary_page_offset)."""
    if len(b) < 12 or b[:4] != b"PAR1" or b[-4:] != b"PAR1":
        raise Unsupported("not a Parquet file")
    n = int.from_bytes(b[-8:-4], "little")
    r = _Thrift(b, len(b) - 8 - n)
    meta = {"num_rows": 0, "schema": [], "row_groups": []}

    def schema_elem():
        e = {"type": -1, "rep": 0, "name": b"", "children": 0, "conv": -1}
        keys = {1: "type", 3: "rep", 5: "children", 6: "conv"}

        def f(i, t):
            if i in keys and t == 5:
                e[keys[i]] = r.zigzag()
            elif i == 4 and t == 8:
                e["name"] = r.binary()
            else:
                return False
            return True
        r.struct(f)
        return e

    def column_meta():
        c = {"codec": 0, "num_values": 0, "data": -1, "dict": -1}

        def f(i, t):
            if i == 4 and t == 5:
                c["codec"] = r.zigzag()
            elif i == 5 and t == 6:
                c["num_values"] = r.zigzag()
            elif i == 9 and t == 6:
                c["data"] = r.zigzag()
            elif i == 11 and t == 6:
                c["dict"] = r.zigzag()
            else:
                return False
            return True
        r.struct(f)
        return c

    def row_group():
        g = {"num_rows": 0, "columns": []}

        def chunk(i, t):
            if i == 3 and t == 12:
                g["columns"].append(column_meta())
                return True
            return False

        def f(i, t):
            if i == 1 and t == 9:
                et, cnt = r.list_header()
                for _ in range(cnt):
                    r.struct(chunk)
            elif i == 3 and t == 6:
                g["num_rows"] = r.zigzag()
            else:
                return False
            return True
        r.struct(f)
        return g

    def top(i, t):
        if i == 2 and t == 9:
            _, cnt = r.list_header()
            meta["schema"] = [schema_elem() for _ in range(cnt)]
        elif i == 3 and t == 6:
            meta["num_rows"] = r.zigzag()
        elif i == 4 and t == 9:
            _, cnt = r.list_header()
            meta["row_groups"] = [row_group() for _ in range(cnt)]
        else:
            return False
        return True
    r.last = [0]
    while True:
        f = r.field()
        if f is None:
            break
        if not top(*f):
            r.skip(f[1])
    sch = meta["schema"]
    if not sch or sch[0]["children"] != len(sch) - 1 or any(e["children"] for e in sch[1:]):
        raise Unsupported("nested schema")
    meta["leaves"] = [(e["name"].decode(), e["type"], e["rep"], e["conv"]) for e in sch[1:]]
    return meta


def read_page_header(b: bytes, at: int) -> dict:
    r = _Thrift(b, at)
    h = {"type": -1, "usize": 0, "csize": 0, "num_values": 0, "encoding": -1, "def_encoding": -1, "def_bytes": 0,
         "rep_bytes": 0, "v2_compressed": True}

    def sub(fields):
        def f(i, t):
            if i in fields and t == 5:
                h[fields[i]] = r.zigzag()
            elif fields is V2 and i == 7 and t in (1, 2):
                h["v2_compressed"] = t == 1
            else:
                return False
            return True
        return f
    V1 = {1: "num_values", 2: "encoding", 3: "def_encoding"}
    V2 = {1: "num_values", 4: "encoding", 5: "def_bytes", 6: "rep_bytes"}
    DICT = {1: "num_values", 2: "encoding"}

    def top(i, t):
        if i in (1, 2, 3) and t == 5:
            h[{1: "type", 2: "usize", 3: "csize"}[i]] = r.zigzag()
        elif i == 5 and t == 12:
            r.struct(sub(V1))
        elif i == 7 and t == 12:
            r.struct(sub(DICT))
        elif i == 8 and t == 12:
            r.struct(sub(V2))
        else:
            return False
        return True
    r.struct(top)
    h["header_bytes"] = r.p - at
    return h


def snappy_decompress(data: bytes) -> bytes:
    """The raw Snappy format: a varint length, then literals and back-references."""
    r = _Thrift(data, 0)
    n = r.varint()
    out = bytearray()
    p = r.p
    while p < len(data):
        tag = data[p]
        kind = tag & 3
        if kind == 0:
            ln = tag >> 2
            if ln < 60:
                p += 1
            else:
                k = ln - 59
                ln = int.from_bytes(data[p + 1:p + 1 + k], "little")
                p += 1 + k
            ln += 1
            out += data[p:p + ln]
            p += ln
            continue
        if kind == 1:
            ln, off = 4 + ((tag >> 2) & 7), ((tag >> 5) << 8) | data[p + 1]
            p += 2
        elif kind == 2:
            ln, off = 1 + (tag >> 2), int.from_bytes(data[p + 1:p + 3], "little")
            p += 3
        else:
            ln, off = 1 + (tag >> 2), int.from_bytes(data[p + 1:p + 5], "little")
            p += 5
        if off == 0 or off > len(out):
            raise Unsupported("snappy: bad offset")
        for _ in range(ln):
            out.append(out[-off])
    if len(out) != n:
        raise Unsupported("snappy: length mismatch")
    return bytes(out)


def hybrid(buf: bytes, pos: int, end: int, bw: int, count: int) -> np.ndarray:
    """count values of the RLE / bit-packed hybrid of bit width bw from buf[pos:end]."""
    out = np.zeros(count, dtype=np.int64)
    k = 0
    r = _Thrift(buf, pos)
    vb = (bw + 7) // 8
    while k < count:
        if r.p >= end:
            raise Unsupported("hybrid: runs end early")
        h = r.varint()
        if h & 1:
            groups = h >> 1
            nbytes = groups * bw
            raw = np.frombuffer(buf[r.p:r.p + nbytes], dtype=np.uint8)
            r.p += nbytes
            m = min(groups * 8, count - k)
            if bw:
                bits = np.unpackbits(raw, bitorder="little")[:groups * 8 * bw].reshape(-1, bw).astype(np.int64)
                vals = (bits << np.arange(bw, dtype=np.int64)).sum(axis=1)
                out[k:k + m] = vals[:m]
            k += m
        else:
            m = min(h >> 1, count - k)
            v = int.from_bytes(buf[r.p:r.p + vb], "little")
            r.p += vb
            out[k:k + m] = v
            k += m
    return out


def scan(b: bytes, projections: Sequence[int], max_row_groups: Optional[int] = None):
    """The scanned frame: one OColumn per projected leaf, every column with a mask (the first
    max_row_groups row groups only, when given: a bounded sample)."""
    from . import make_column
    meta = read_footer(b)
    if max_row_groups is not None:
        meta["row_groups"] = meta["row_groups"][:max_row_groups]
    cols = []
    for c in projections:
        name, ptype, rep, conv = meta["leaves"][c]
        if ptype not in _NP or (ptype == 1 and conv not in (-1, 6)) or (ptype == 2 and conv not in (-1, 9)) or rep == 2:
            raise Unsupported(f"leaf {name}")
        dt = {1: fe.GDF_DATE32 if conv == 6 else fe.GDF_INT32, 2: fe.GDF_DATE64 if conv == 9 else fe.GDF_INT64,
              4: fe.GDF_FLOAT32, 5: fe.GDF_FLOAT64}[ptype]
        npd = np.dtype(_NP[ptype])
        vals, valid = [], []
        for g in meta["row_groups"]:
            cc = g["columns"][c]
            if cc["codec"] not in (0, 1):
                raise Unsupported("codec")
            at = min(cc["dict"], cc["data"]) if cc["dict"] >= 4 else cc["data"]
            seen, dictionary = 0, None
            while seen < cc["num_values"]:
                h = read_page_header(b, at)
                data = at + h["header_bytes"]
                body = b[data:data + h["csize"]]
                at = data + h["csize"]
                if h["type"] not in (0, 2, 3):
                    continue
                v2 = h["type"] == 3
                raw = h["def_bytes"] + h["rep_bytes"] if v2 else 0
                if cc["codec"] == 1 and (not v2 or h["v2_compressed"]):
                    body = body[:raw] + snappy_decompress(body[raw:])
                if h["type"] == 2:
                    dictionary = np.frombuffer(body[:h["num_values"] * npd.itemsize], dtype=npd)
                    continue
                nv = h["num_values"]
                seen += nv
                if rep == 1:
                    if v2:
                        lev_end, p = h["def_bytes"], h["def_bytes"]
                        lev = hybrid(body, 0, lev_end, 1, nv)
                    else:
                        ln = int.from_bytes(body[:4], "little")
                        lev = hybrid(body, 4, 4 + ln, 1, nv)
                        p = 4 + ln
                    m = lev.astype(bool)
                else:
                    m = np.ones(nv, dtype=bool)
                    p = raw if v2 else 0
                k = int(m.sum())
                if h["encoding"] == 0:
                    present = np.frombuffer(body[p:p + k * npd.itemsize], dtype=npd)
                elif h["encoding"] in (2, 8):
                    ix = hybrid(body, p + 1, len(body), body[p], k)
                    present = dictionary[ix]
                else:
                    raise Unsupported("encoding")
                v = np.zeros(nv, dtype=npd)
                v[m] = present
                vals.append(v)
                valid.append(m)
        v = np.concatenate(vals) if vals else np.zeros(0, dtype=npd)
        m = np.concatenate(valid) if valid else np.zeros(0, dtype=bool)
        cols.append(make_column(v, dt, m))
    return cols


def scan_filter(b: bytes, projections: Sequence[int], filter_query_part: Optional[str] = None,
                max_row_groups: Optional[int] = None, nthreads: int = 1):
    """BindableTableScan followed by its LogicalFilter (None: the scan alone)."""
    from . import process_filter
    cols = scan(b, projections, max_row_groups)
    return cols if filter_query_part is None else process_filter(cols, filter_query_part, nthreads=nthreads)
