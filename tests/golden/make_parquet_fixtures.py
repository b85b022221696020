"""Writes the Parquet fixtures of tests/test_gpu_parquet.py with pyarrow (a second, independent
writer beside ralgpu.workloads.parquet_bytes), and the column values each file holds as .npz.
Run from the repository root: python tests/golden/make_parquet_fixtures.py"""
import os

import numpy as np
import pyarrow as pa
import pyarrow.parquet as pq

HERE = os.path.dirname(os.path.abspath(__file__))


def table(n, seed, low_card=False):
    """Six leaves: a int32 (8% null), b int64, c float32 (30% null), d float64, e date32 (2% null),
    f timestamp[ms]; low_card draws each from a few values (dictionary pages stay in use)."""
    rng = np.random.default_rng(seed)

    def opt(v, rate):
        m = rng.random(n) >= rate
        return np.where(m, v, 0).astype(v.dtype), m

    def pick(vals, dtype):
        return np.asarray(vals, dtype=dtype)[rng.integers(0, len(vals), n)]

    if low_card:
        a, ma = opt(pick(range(-50, 50), np.int32), 0.08)
        b = pick([k * 1_000_003 for k in range(1000)], np.int64)
        c, mc = opt(pick(rng.standard_normal(20), np.float32), 0.3)
        d = pick(rng.uniform(-1e3, 1e3, 50), np.float64)
        e, me = opt(pick(range(9000, 9100), np.int32), 0.02)
        f = pick(rng.integers(0, 2 * 10**12, 30), np.int64)
    else:
        a, ma = opt(rng.integers(-10**6, 10**6, n).astype(np.int32), 0.08)
        b = rng.integers(-(1 << 50), 1 << 50, n).astype(np.int64)
        c, mc = opt(rng.standard_normal(n).astype(np.float32), 0.3)
        d = rng.uniform(-1e3, 1e3, n)
        e, me = opt(rng.integers(8000, 11000, n).astype(np.int32), 0.02)
        f = rng.integers(0, 2 * 10**12, n).astype(np.int64)
    g = np.array([f"s{k % 7}" for k in range(n)])
    t = pa.table({"a": pa.array(a, mask=~ma), "b": pa.array(b), "c": pa.array(c, mask=~mc), "d": pa.array(d),
                  "e": pa.array(e, mask=~me).cast(pa.date32()), "f": pa.array(f).cast(pa.timestamp("ms")),
                  "g": pa.array(g)})
    t = t.cast(pa.schema([pa.field("a", pa.int32()), pa.field("b", pa.int64(), nullable=False),
                          pa.field("c", pa.float32()), pa.field("d", pa.float64(), nullable=False),
                          pa.field("e", pa.date32()), pa.field("f", pa.timestamp("ms"), nullable=False),
                          pa.field("g", pa.string(), nullable=False)]))
    vals = dict(a=a, a_valid=ma, b=b, c=c, c_valid=mc, d=d, e=e, e_valid=me, f=f)
    return t, vals


# name: (rows, seed, low cardinality, write_table options)
FILES = {
    "parquet_plain": (3000, 3, False, dict(compression="NONE", use_dictionary=False, data_page_version="1.0",
                                           row_group_size=1200, data_page_size=1024)),
    "parquet_snappy": (3000, 4, False, dict(compression="SNAPPY", use_dictionary=False, data_page_version="1.0",
                                            row_group_size=1200, data_page_size=1024)),
    "parquet_dictionary": (3000, 5, True, dict(compression="NONE", use_dictionary=True, data_page_version="1.0",
                                               row_group_size=1200, data_page_size=1024)),
    "parquet_dict_fallback": (3000, 6, False, dict(compression="NONE", use_dictionary=True, data_page_version="1.0",
                                                   dictionary_pagesize_limit=2048, data_page_size=1024)),
    "parquet_v2": (3000, 7, False, dict(compression="NONE", use_dictionary=False, data_page_version="2.0",
                                        row_group_size=1200, data_page_size=1024)),
    "parquet_v2_snappy_dict": (3000, 8, True, dict(compression="SNAPPY", use_dictionary=True, data_page_version="2.0",
                                                   row_group_size=1500, data_page_size=2048)),
    "parquet_defaults": (3000, 9, True, dict()),
    "parquet_gzip": (300, 10, False, dict(compression="GZIP", use_dictionary=False)),
    "parquet_delta": (300, 11, False, dict(compression="NONE", use_dictionary=False,
                                           column_encoding={"b": "DELTA_BINARY_PACKED"})),
}


def main():
    for name, (n, seed, low, opts) in FILES.items():
        t, vals = table(n, seed, low)
        pq.write_table(t, os.path.join(HERE, name + ".parquet"), write_statistics=False, **opts)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **vals)


if __name__ == "__main__":
    main()
