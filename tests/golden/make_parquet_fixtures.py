"""Writes the Parquet fixtures of tests/test_gpu_parquet.py with pyarrow (a second, independent
writer beside ralgpu.workloads.parquet_bytes), and the column values each file holds as .npz.
Run from the repository root: python tests/golden/make_parquet_fixtures.py"""
import os

import numpy as np
import pyarrow as pa
import pyarrow.parquet as pq

HERE = os.path.dirname(os.path.abspath(__file__))


def table(n, seed):
    rng = np.random.default_rng(seed)

    def opt(v, rate):
        m = rng.random(n) >= rate
        return np.where(m, v, 0).astype(v.dtype), m

    a, ma = opt(rng.integers(-10**6, 10**6, n).astype(np.int32), 0.08)
    b = rng.integers(-(1 << 50), 1 << 50, n).astype(np.int64)
    c, mc = opt(rng.standard_normal(n).astype(np.float32), 0.3)
    d = rng.uniform(-1e3, 1e3, n)
    e, me = opt(rng.integers(8000, 11000, n).astype(np.int32), 0.02)
    f = rng.integers(0, 2 * 10**12, n).astype(np.int64)
    t = pa.table({"a": pa.array(a, mask=~ma), "b": pa.array(b), "c": pa.array(c, mask=~mc), "d": pa.array(d),
                  "e": pa.array(e, mask=~me).cast(pa.date32()), "f": pa.array(f).cast(pa.timestamp("ms"))})
    t = t.cast(pa.schema([pa.field("a", pa.int32()), pa.field("b", pa.int64(), nullable=False),
                          pa.field("c", pa.float32()), pa.field("d", pa.float64(), nullable=False),
                          pa.field("e", pa.date32()), pa.field("f", pa.timestamp("ms"), nullable=False)]))
    vals = dict(a=a, a_valid=ma, b=b, c=c, c_valid=mc, d=d, e=e, e_valid=me, f=f)
    return t, vals


def main():
    t, vals = table(3000, 3)
    pq.write_table(t, os.path.join(HERE, "parquet_plain.parquet"), compression="NONE", use_dictionary=False,
                   data_page_version="1.0", write_statistics=False, row_group_size=1200, data_page_size=1024)
    np.savez(os.path.join(HERE, "parquet_plain.npz"), **vals)
    small, _ = table(300, 4)
    pq.write_table(small, os.path.join(HERE, "parquet_snappy.parquet"), compression="SNAPPY", use_dictionary=False,
                   data_page_version="1.0")
    pq.write_table(small, os.path.join(HERE, "parquet_dictionary.parquet"), compression="NONE", use_dictionary=True,
                   data_page_version="1.0")


if __name__ == "__main__":
    main()
