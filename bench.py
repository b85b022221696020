"""Benchmark of the GB300 expression path (one JSON line on rank 0).

Default workload: fused_project — the 200M-row, 12-op fused projection with 5
nullable inputs and 3 outputs (f1, f2 float64; i1 int64), evaluated by
ral_perform_operation_async on HBM-resident columns.  Other workloads:
  --workload plain_vm          1M-row filter + project (fused)
  --workload filter_gather     500M-row filter + compaction + gather, --selectivity 0.01/0.5/0.99
  --workload filter_project    200M-row fused filter + project: the fused_project columns and its
                               projection (as RexNode text) behind a filter on k, --selectivity s
  --workload batched           256 programs of 4-48 ops over tables of log-uniform [1e3, 5e7] rows,
                               all in one persistent launch replayed as a CUDA graph, against the
                               same 256 programs as plain synchronous perform_operation calls
  --workload served            Poisson request loop over 24 resident tables (log-uniform [1e4, 1e8]
                               rows) and 96 prepared filter + project queries of 4-32 ops, at 5
                               rates, ~50k requests: p50 / p99 latency and rows/s of the served
                               (continuously batched) loop against serial plain execution
  --workload scan_filter       20M-row lineitem-like '|'-delimited text (1.3 GB) scanned and
                               filtered by TPC-H Q6's conditions in one fused kernel

value     rows/s over the timed steps (inputs resident in HBM; every input > L2, so no flush)
e2e       same metric through the C ABI with host buffers: pinned H2D of the inputs and D2H of
          the outputs inside the timed region
roofline  algorithmic bytes / kernel time of the dominant kernel vs MEASURED_PEAKS.json hbm_gbs
cpu_baseline  the CPU oracle (a row-by-row port of the reference interpreter) on all host cores,
          timed on a bounded sample of the same workload

--impl reference times the reference's CPU implementation of the path: the reference's
interpreter only exists as GPU code built against cudf, which is not available, so the oracle
port stands in (kind "port").  Multi-GPU: replicas (each rank runs its own copy of the workload).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "blazingdb-ral_gb300"))
sys.path.insert(0, ROOT)

METRIC = "filter+project rows/s & HBM GB/s vs 8 TB/s; batched/served rows/s, p99 vs plain"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def load_traffic(key):
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get(key)
    return None


# GB300's FP64 pipe: two thread instructions per clock per SM (from the counters: C2's 100M FP64
# instructions ran at 63% pipe activity in 261 us at 2070 MHz = 1.93 per clock per SM)
FP64_PER_CLOCK_PER_SM = 2.0
SMS = 152


def batch_mix_meta(n_programs, seed):
    """Per program of the batched mix, without a GPU: rows and algorithmic bytes per row."""
    import ralgpu as R
    from ralgpu import dtypes as D
    from ralgpu import workloads as W
    out = []
    for t in W.batched_mix(n_programs, seed=seed):
        pp = R.parse_project_plan(t.dtypes, t.project)
        bpr = 0.0
        for c in pp["input_columns"]:
            bpr += D.WIDTH[t.dtypes[c]] + (1 / 8 if t.null_rates[c] > 0 else 0)
        bpr += sum(D.WIDTH[dt] + 1 / 8 for dt in pp["evaluated_dtypes"])
        out.append({"rows": int(t.rows), "bytes_per_row": bpr})
    return out


def floor_table_from_ncu(csv_path, n_programs, seed, cap):
    """profiles/batch_mix_fp64.json from an ncu CSV of the mix's plain calls over tables capped at
    `cap` rows (one ral_eval launch per program, in program order): FP64 and all thread
    instructions per row of every program."""
    import csv
    rows = [r for r in csv.reader(open(csv_path)) if len(r) > 14 and r[0].isdigit()]
    by = {}
    for r in rows:
        by.setdefault(int(r[0]), {})[r[12]] = float(r[14].replace(",", ""))
    ids = sorted(by)
    meta = batch_mix_meta(n_programs, seed)
    if len(ids) != len(meta):
        raise SystemExit(f"{len(ids)} launches in {csv_path} for {len(meta)} programs")
    progs = []
    for i, m in zip(ids, meta):
        rc = min(m["rows"], cap)
        progs.append({"rows": m["rows"], "bytes_per_row": round(m["bytes_per_row"], 4),
                      "fp64_per_row": by[i]["sm__thread_inst_executed_pipe_fp64_pred_on.sum"] / rc,
                      "inst_per_row": by[i]["smsp__thread_inst_executed.sum"] / rc})
    return {"what": "per program of the 256-program batched mix (seed %d), from plain calls over the first %d rows "
                    "of each table" % (seed, cap),
            "command": "ncu --metrics sm__thread_inst_executed_pipe_fp64_pred_on.sum,smsp__thread_inst_executed.sum,"
                       "gpu__time_duration.sum --clock-control none -k regex:ral_eval -s 512 -c 256 --csv --log-file "
                       "batch_fp64.csv python bench.py --workload batched --max-rows %d --steps 1 --warmup 1 "
                       "--plain-steps 1 --capped-rows 0 --no-autotune" % cap,
            "programs": progs}


def batch_floor(table, sm_mhz, peak_gbs):
    """The mix's floor: the FP64-pipe time of its instructions and the HBM time of its bytes, for
    the whole mix overlapped (a batch) and program by program (plain calls, one after another)."""
    rate = FP64_PER_CLOCK_PER_SM * SMS * sm_mhz * 1e6
    fp = [p["rows"] * p["fp64_per_row"] / rate for p in table["programs"]]
    hb = [p["rows"] * p["bytes_per_row"] / (peak_gbs * 1e9) for p in table["programs"]]
    return {"fp64_ms": sum(fp) * 1e3, "hbm_ms": sum(hb) * 1e3,
            "floor_ms": max(sum(fp), sum(hb)) * 1e3,
            "per_program_floor_ms": sum(max(a, b) for a, b in zip(fp, hb)) * 1e3,
            "fp64_rate": f"{FP64_PER_CLOCK_PER_SM} per clock per SM x {SMS} SMs x {sm_mhz:.0f} MHz",
            "source": "profiles/batch_mix_fp64.json"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 20 ms; only samples that arrive
    inside the timed window [mark_start, mark_end] are kept."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, bufsize=1)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(1.0)   # let nvidia-smi start emitting before the timed region
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def mark_start(self):
        self.t0 = time.monotonic()

    def mark_end(self):
        self.t1 = time.monotonic()

    def stop(self):
        """Ends sampling; summary of the window [mark_start, mark_end]."""
        if self.proc is not None:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return self.window(self.t0, self.t1)

    def window(self, t0, t1):
        """Median SM clock, max clock and throttle reasons of the samples taken in [t0, t1]."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        lines = list(self.lines)
        inside = [ln for t, ln in lines if t0 is not None and t0 <= t <= t1 + 0.05]
        window = "timed region"
        if not inside:
            # a very short timed region: take the samples nearest to it
            near = sorted(lines, key=lambda x: abs(x[0] - (t0 or 0)))[:3]
            inside = [ln for _, ln in near]
            window = "nearest samples (timed region shorter than the sampling period)"
        sm, smax, power, reasons = [], [], [], set()
        for ln in inside:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(self.NAMES, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "window": window,
                "power_w_max": max(power) if power else None}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        # replicas only exchange their timings: NCCL on GPUs, gloo for the CPU reference arm (and
        # for CPU tests of this coordination, RAL_DIST_BACKEND=gloo)
        backend = os.environ.get("RAL_DIST_BACKEND") or ("nccl" if args.impl != "reference" else "gloo")
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, ms_per_step):
    """Whole-job throughput of N replicas: every rank's units over the slowest rank's time."""
    return world * units_per_rank / (ms_per_step / 1e3)


# ---- CPU oracle timing --------------------------------------------------------------------------

def cpu_fused_project(rows: int, threads: int):
    import numpy as np
    import oracle as O
    from oracle import frontend as fe
    from ralgpu import workloads as W
    spec = W.fused_project_program()
    inputs = W.fused_project_host(rows, seed=99)
    ins = [O.make_column(v, t, m) for t, v, m in inputs]
    outs = [O.alloc_column(t, rows) for t in spec.output_dtypes]
    ls = [fe.Scalar(*s) for s in spec.lscalars]
    rs = [fe.Scalar(*s) for s in spec.rscalars]
    t0 = time.perf_counter()
    O.perform_operation(outs, ins, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops, ls, rs,
                        nthreads=threads)
    return time.perf_counter() - t0


def cpu_plain_vm(rows: int, threads: int):
    import oracle as O
    from ralgpu import workloads as W
    spec = W.plain_vm_host(rows, seed=99)
    frame = [O.make_column(v, t, m) for t, v, m in spec]
    t0 = time.perf_counter()
    f = O.process_filter(frame, W.PLAIN_VM_FILTER, nthreads=threads)
    O.execute_project_plan(f, W.PLAIN_VM_PROJECT, nthreads=threads)
    return time.perf_counter() - t0


def cpu_filter_gather(rows: int, threads: int, selectivity: float):
    import oracle as O
    from ralgpu import workloads as W
    spec = W.filter_gather_host(rows, seed=99)
    frame = [O.make_column(v, t, m) for t, v, m in spec]
    t0 = time.perf_counter()
    O.process_filter(frame, W.filter_gather_query(selectivity), nthreads=threads)
    return time.perf_counter() - t0


def cpu_filter_project(rows: int, threads: int, selectivity: float):
    import oracle as O
    from ralgpu import workloads as W
    frame = [O.make_column(v, t, m) for t, v, m in W.fused_project_host(rows, seed=99)]
    t0 = time.perf_counter()
    f = O.process_filter(frame, W.filter_project_filter(selectivity), nthreads=threads)
    O.execute_project_plan(f, W.FILTER_PROJECT_PROJECT, nthreads=threads)
    return time.perf_counter() - t0


def _scan_chunk(args):
    """A process-pool task: the oracle's scan of text rows [r0, r1) of the fixed-width table."""
    text, proj = args
    from oracle import textscan as T
    from ralgpu import workloads as W
    return [(c.data[:c.size].copy(), c.valid_bools().copy()) for c in T.scan(text, W.TEXT_DTYPES, proj)]


_SCAN_POOL = None


def cpu_scan_filter(rows, threads):
    """The oracle's text scan (one process per thread, each a slice of the rows) and its filter;
    returns seconds.  The pool starts from a clean interpreter (spawn) and is kept between calls."""
    import multiprocessing as mp
    import numpy as np
    import oracle as O
    from ralgpu import workloads as W
    global _SCAN_POOL
    text = W.text_table(rows, seed=W.SEED + 5)
    w = W.TEXT_ROW_BYTES
    per = (rows + threads - 1) // threads
    tasks = [(text[k * per * w:min(rows, (k + 1) * per) * w], W.TEXT_PROJECTIONS) for k in range(threads) if k * per < rows]
    if threads > 1 and _SCAN_POOL is None:
        _SCAN_POOL = mp.get_context("spawn").Pool(threads)
        _SCAN_POOL.map(_scan_chunk, [(b"1|2|3|4|5|6|1995-01-01|1995-01-01\n", W.TEXT_PROJECTIONS)] * threads)
    t0 = time.perf_counter()
    parts = _SCAN_POOL.map(_scan_chunk, tasks) if threads > 1 else [_scan_chunk(t) for t in tasks]
    frame = []
    for k, c in enumerate(W.TEXT_PROJECTIONS):
        v = np.concatenate([p[k][0] for p in parts])
        m = np.concatenate([p[k][1] for p in parts])
        frame.append(O.make_column(v, W.TEXT_DTYPES[c], m))
    O.process_filter(frame, W.TEXT_FILTER, nthreads=threads)
    return time.perf_counter() - t0


def cpu_time(workload, rows, threads, selectivity):
    if workload == "scan_filter":
        return cpu_scan_filter(rows, threads)
    if workload == "gather":
        return cpu_gather(rows, threads)
    if workload == "fused_project":
        return cpu_fused_project(rows, threads)
    if workload == "filter_project":
        return cpu_filter_project(rows, threads, selectivity)
    if workload == "plain_vm":
        return cpu_plain_vm(rows, threads)
    return cpu_filter_gather(rows, threads, selectivity)


def cpu_model() -> str:
    """The host CPU's model name (lscpu), for the record of where the CPU figures were taken."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_baseline(workload, full_rows, selectivity, budget_s=12.0, single_budget_s=4.0):
    """rows/s of the oracle on all cores over a bounded sample sized for about budget_s of work, and
    on one thread over a sample sized for about single_budget_s."""
    threads = os.cpu_count() or 1
    # the text scan's oracle parses in Python: a smaller first probe
    probe = min(full_rows, 200_000 if workload == "scan_filter" else 2_000_000)
    dt = cpu_time(workload, probe, threads, selectivity)
    rate = probe / max(dt, 1e-9)
    rows = int(min(full_rows, max(probe, rate * budget_s / 3)))
    times = [cpu_time(workload, rows, threads, selectivity) for _ in range(3)]
    t = statistics.median(times)
    out = {"value": rows / t, "unit": "rows/s", "cores": threads, "kind": "port",
           "sample": f"{rows} of {full_rows} rows, median of 3 runs, {threads} threads",
           "cpu_model": cpu_model()}
    if single_budget_s > 0:
        p1 = min(full_rows, 20_000 if workload == "scan_filter" else 200_000)
        d1 = cpu_time(workload, p1, 1, selectivity)
        r1 = int(min(full_rows, max(p1, (p1 / max(d1, 1e-9)) * single_budget_s / 3)))
        t1 = statistics.median([cpu_time(workload, r1, 1, selectivity) for _ in range(3)])
        out["single_thread"] = {"value": r1 / t1, "unit": "rows/s", "cores": 1,
                                "sample": f"{r1} of {full_rows} rows, median of 3 runs, 1 thread"}
    return out


def cpu_batched(threads: int, n_programs: int, rows_cap: int, seed: int = 20261203):
    """Oracle over the first n_programs of the batched mix, each table capped at rows_cap rows;
    returns (rows, seconds)."""
    import oracle as O
    from oracle import frontend as fe
    import ralgpu as R
    from ralgpu import workloads as W
    mix = W.batched_mix(256, seed=seed)[:n_programs]
    jobs = []
    for t in mix:
        pp = R.parse_project_plan(t.dtypes, t.project)
        host = W.batched_table_host(t, rows=min(t.rows, rows_cap))
        ins = [O.make_column(host[c][1], host[c][0], host[c][2]) for c in pp["input_columns"]]
        n = ins[0].size
        outs = [O.alloc_column(dt, n) for dt in pp["evaluated_dtypes"]]
        jobs.append((pp, ins, outs, n))
    t0 = time.perf_counter()
    rows = 0
    for pp, ins, outs, n in jobs:
        O.perform_operation(outs, ins, pp["left"], pp["right"], pp["outputs"], pp["final_output_positions"],
                            pp["operators"], pp["unary_operators"],
                            [fe.Scalar(x.dtype, x.value, x.is_valid) for x in pp["left_scalars"]],
                            [fe.Scalar(x.dtype, x.value, x.is_valid) for x in pp["right_scalars"]], nthreads=threads)
        rows += n
    return rows, time.perf_counter() - t0


def cpu_served(threads: int, n_queries: int, rows_cap: int, seed: int = 20261203):
    """Oracle filter + project over the first n_queries of the served workload, tables capped at
    rows_cap rows; returns (rows scanned, seconds)."""
    import oracle as O
    from ralgpu import workloads as W
    tabs = W.served_tables(24, seed=seed)
    qs = W.served_queries(tabs, 96, seed=seed)[:n_queries]
    frames = {}
    for q in qs:
        if q.table not in frames:
            host = W.served_table_host(tabs[q.table], rows=min(tabs[q.table].rows, rows_cap))
            frames[q.table] = [O.make_column(v, t, m) for t, v, m in host]
    t0 = time.perf_counter()
    rows = 0
    for q in qs:
        f = O.process_filter(frames[q.table], q.filter, nthreads=threads)
        O.execute_project_plan(f, q.project, nthreads=threads)
        rows += frames[q.table][0].size
    return rows, time.perf_counter() - t0


# ---- GPU workloads --------------------------------------------------------------------------------

DEFAULT_ROWS = {"fused_project": 200_000_000, "plain_vm": 1_000_000, "filter_gather": 500_000_000,
                "filter_project": 200_000_000, "gather": 200_000_000, "scan_filter": 20_000_000,
                "parquet_filter": 20_000_000, "parquet_dict_filter": 20_000_000}


def workload_config(workload, n, selectivity, world=1):
    """The `config` object of a workload: the same dict on both arms of the benchmark."""
    if workload == "fused_project":
        cfg = {"workload": "fused_project", "rows": n, "inputs": "a,b int64; x,y float64; k int32; 5% nulls",
               "program_ops": 12, "outputs": "f1,f2 float64; i1 int64",
               "l2": "inputs (12.2 GB at 200M rows) exceed L2; no flush"}
    elif workload == "filter_project":
        cfg = {"workload": "filter_project", "rows": n, "selectivity": selectivity,
               "filter": f"k < {int(round(1000 * selectivity))}", "project": "f1, f2, i1 of the 12-op program",
               "inputs": "a,b int64; x,y float64; k int32; 5% nulls", "fused": "filter+project in one kernel",
               "l2": "inputs exceed L2; no flush"}
    elif workload == "gather":
        cfg = {"workload": "gather", "rows": n, "pattern": selectivity if isinstance(selectivity, str) else "permutation",
               "columns": "int32, int64, float32, float64, date32, bool8; 5% nulls", "index": "int32",
               "api": "ral_materialize_columns (all columns in one kernel)",
               "l2": "columns (5.8 GB at 200M rows) exceed L2; no flush"}
    elif workload in PARQUET_WORKLOADS:
        from ralgpu import workloads as W
        dictionary = workload == "parquet_dict_filter"
        cfg = {"workload": workload, "rows": n,
               "table": "the lineitem-like table as Parquet: 8 required columns, uncompressed "
                        + ("dictionary-encoded v1 pages (a chunk of at most 65,536 distinct values as a PLAIN "
                           "dictionary and RLE_DICTIONARY pages, others PLAIN)" if dictionary else "PLAIN v1 pages")
                        + ", 1Mi-row row groups, in page-locked host memory",
               "scan": f"BindableTableScan projects={W.TEXT_PROJECTIONS}", "filter": "TPC-H Q6's conditions",
               "fused": "the projected pages read in place from page-locked host memory"
                        + (", dictionary indices decoded by one block per page" if dictionary else "")
                        + ", the page-value kernel (a block per 8192-row item of a page), then the fused filter kernel",
               "l2": "decoded columns (560 MB at 20M rows) exceed L2; no flush"}
    elif workload == "scan_filter":
        from ralgpu import workloads as W
        cfg = {"workload": "scan_filter", "rows": n, "text_bytes": n * W.TEXT_ROW_BYTES,
               "table": "lineitem-like '|'-delimited text: orderkey int64, partkey int32, quantity int32, "
                        "extendedprice float64, discount float64, tax float32, shipdate date64, commitdate date32",
               "scan": f"BindableTableScan projects={W.TEXT_PROJECTIONS}", "filter": "TPC-H Q6's conditions",
               "fused": "parse + filter + compaction in one kernel (after a line index)",
               "l2": "text (1.3 GB at 20M rows) exceeds L2; no flush"}
    elif workload == "plain_vm":
        cfg = {"workload": "plain_vm", "rows": n, "filter": "((c2>=24 AND c1<0.05) OR c0%7=3) AND c3<1200",
               "project": "c1*(1-c1)+c2", "fused": "filter+project in one kernel",
               "l2": "1M rows (24 MB) fit in L2: per-call latency bound"}
    else:
        from ralgpu import workloads as W
        cfg = {"workload": "filter_gather", "rows": n, "selectivity": selectivity,
               "predicate": f"<($0, {W.FILTER_THRESHOLDS[selectivity]})", "gathered_columns": 6,
               "l2": "inputs exceed L2; no flush"}
    cfg["parallelism"] = f"replicas x{world}"
    return cfg


def scan_filter_setup(n, device):
    """The lineitem-like text table in device memory, its ground-truth column values, and one step:
    ral_text_scan_filter of TPC-H Q6's conditions over the scan of quantity, extendedprice, discount
    and shipdate, into outputs sized for every row."""
    import ctypes
    import torch
    import ralgpu as R
    from ralgpu import dtypes as D
    from ralgpu import workloads as W
    L = R.lib()
    text, values = W.text_table(n, seed=W.SEED, values=True)
    host = torch.frombuffer(bytearray(text), dtype=torch.uint8).pin_memory()
    dev = host.to(device)
    proj = W.TEXT_PROJECTIONS
    outs = [R.Column.empty(W.TEXT_DTYPES[c], n, with_valid=True, device=device) for c in proj]
    oa, os_ = _colarray(outs)
    fd = (ctypes.c_int32 * len(W.TEXT_DTYPES))(*W.TEXT_DTYPES)
    pr = (ctypes.c_int32 * len(proj))(*proj)
    nout = ctypes.c_int32(0)
    fq = W.TEXT_FILTER.encode()

    def scan(ptr, from_host=False):
        for st in os_:  # the outputs' capacity (a call leaves size = rows kept)
            st.size = n
        fn = L.ral_text_scan_filter_host if from_host else L.ral_text_scan_filter
        rc = fn(ctypes.c_void_p(ptr), len(text), b"|", b"\n", 0, fd, len(fd), pr, len(pr), fq,
                ctypes.cast(oa, ctypes.c_void_p), ctypes.byref(nout))
        if rc:
            raise RuntimeError(L.ral_last_error().decode())

    def step(stream):
        scan(dev.data_ptr())

    def alg_bytes():
        k = nout.value
        return len(text) + k * sum(D.WIDTH[W.TEXT_DTYPES[c]] + 1 / 8 for c in proj)

    return dict(step=step, scan=scan, alg_bytes_fn=alg_bytes, nout=nout, outs=outs, out_structs=os_, values=values,
                host_text=host, dev_text=dev, text_bytes=len(text), cols=[R.Column(dev, None, D.GDF_INT8, len(text))])


PARQUET_WORKLOADS = ("parquet_filter", "parquet_dict_filter")


def parquet_filter_setup(n, device, dictionary=False):
    """The lineitem-like table as a Parquet file in page-locked host memory, and one step:
    ral_parquet_scan_filter of TPC-H Q6's conditions over the scan of quantity, extendedprice,
    discount and shipdate (the projected pages read in place over the host link, decoded, filtered)."""
    import ctypes
    import torch
    import ralgpu as R
    from ralgpu import dtypes as D
    from ralgpu import workloads as W
    L = R.lib()
    values = W.lineitem_values(n, W.SEED)
    sizes = []
    blob = W.parquet_bytes([(nm, dt, v, None) for nm, dt, v in zip(W.LINEITEM_NAMES, W.TEXT_DTYPES, values)],
                           dictionary=dictionary, chunk_bytes=sizes)
    host = torch.frombuffer(bytearray(blob), dtype=torch.uint8).pin_memory()
    proj = W.TEXT_PROJECTIONS
    outs = [R.Column.empty(W.TEXT_DTYPES[c], n, with_valid=True, device=device) for c in proj]
    oa, os_ = _colarray(outs)
    pr = (ctypes.c_int32 * len(proj))(*proj)
    nout = ctypes.c_int32(0)
    fq = W.TEXT_FILTER.encode()

    def step(stream):
        for st in os_:  # the outputs' capacity (a call leaves size = rows kept)
            st.size = n
        rc = L.ral_parquet_scan_filter(ctypes.c_void_p(host.data_ptr()), len(blob), pr, len(pr), fq,
                                       ctypes.cast(oa, ctypes.c_void_p), ctypes.byref(nout))
        if rc:
            raise RuntimeError(L.ral_last_error().decode())

    # the bytes that cross the link: the projected leaves' column chunks
    chunk_bytes = sum(b for c, b in sizes if c in proj)

    def alg_bytes():
        k = nout.value
        return chunk_bytes + k * sum(D.WIDTH[W.TEXT_DTYPES[c]] + 1 / 8 for c in proj)

    return dict(step=step, alg_bytes_fn=alg_bytes, nout=nout, outs=outs, out_structs=os_, values=values,
                file_bytes=len(blob), chunk_bytes=chunk_bytes, cols=[R.Column(host, None, D.GDF_INT8, len(blob))],
                blob=blob, rows=n, row_group_rows=1 << 20, row_groups=(n + (1 << 20) - 1) >> 20)


def cpu_parquet(ctx, budget_s=10.0):
    """The oracle's Parquet reader (numpy page decode, oracle/parquet.py) and process_filter on all
    host threads, over the first row groups of the same file: as many as fit the budget."""
    import oracle.parquet as OP
    from ralgpu import workloads as W
    blob = ctx["blob"]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    OP.scan_filter(blob, W.TEXT_PROJECTIONS, W.TEXT_FILTER, max_row_groups=1, nthreads=threads)
    one = max(time.perf_counter() - t0, 1e-3)
    groups = int(max(1, min(ctx["row_groups"], budget_s / one)))
    t0 = time.perf_counter()
    OP.scan_filter(blob, W.TEXT_PROJECTIONS, W.TEXT_FILTER, max_row_groups=groups, nthreads=threads)
    dt = time.perf_counter() - t0
    rows = min(ctx["rows"], groups * ctx["row_group_rows"])
    return {"value": rows / dt, "unit": "rows/s", "cores": threads, "kind": "port",
            "sample": f"first {groups} row groups ({rows} rows): page decode on one thread (numpy), "
                      f"the filter on {threads}", "cpu_model": cpu_model()}


def scan_filter_parity(ctx):
    """The kept rows against the oracle's filter over the values the text spells (the oracle's own
    parse of the same fixed-width fields is checked against those values by the tests)."""
    import numpy as np
    import oracle as O
    from ralgpu import workloads as W
    t0 = time.perf_counter()
    n = len(ctx["values"][0])
    frame = [O.make_column(np.asarray(ctx["values"][c]), W.TEXT_DTYPES[c], np.ones(n, dtype=bool))
             for c in W.TEXT_PROJECTIONS]
    exp = O.process_filter(frame, W.TEXT_FILTER, nthreads=os.cpu_count() or 1)
    stats = {"valid": 0, "data": 0, "rows_out": abs(ctx["nout"].value - exp[0].size), "null_count": 0}
    for g, e in zip(ctx["outs"], exp):
        O.update_null_count(e)
        k = min(g.size, e.size)
        if k:
            _compare(g, 0, k, e, stats)
        stats["null_count"] += abs(g.null_count - e.null_count)
    return {"rows": n, "rows_out": ctx["nout"].value, "mismatches": sum(stats.values()), "detail": stats,
            "checked": "every kept row, bit for bit: data, validity bits, null counts, kept row count and order",
            "seconds": round(time.perf_counter() - t0, 2)}


def scan_filter_e2e(ctx, steps):
    """The text from page-locked host memory: each step hands it to ral_text_scan_filter_host (which
    copies it in pieces, each scanned while the next are copied) and copies the kept rows' columns
    and masks back."""
    import torch
    import ralgpu as R
    host = ctx["host_text"]
    outs = ctx["outs"]
    back = [(torch.empty_like(o.data, device="cpu").pin_memory(), torch.empty_like(o.valid, device="cpu").pin_memory())
            for o in outs]
    stream = torch.cuda.current_stream()

    def one():
        ctx["scan"](host.data_ptr(), from_host=True)
        k = ctx["nout"].value
        for (bd, bv), o in zip(back, outs):
            bd[:k].copy_(o.data[:k], non_blocking=True)
            bv[:(k + 7) // 8].copy_(o.valid[:(k + 7) // 8], non_blocking=True)
        stream.synchronize()
        return k

    one()
    times = []
    k = 0
    for _ in range(max(steps, 5)):
        t0 = time.perf_counter()
        k = one()
        times.append((time.perf_counter() - t0) * 1e3)
    ms = statistics.median(times)
    d2h = sum(k * o.data.element_size() + (k + 7) // 8 for o in outs)
    n = len(ctx["values"][0])
    return {"value": n / (ms / 1e3), "unit": "rows/s", "h2d_bytes_per_step": int(ctx["text_bytes"]),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": ms, "timing": f"median of {len(times)} steps after one",
            "api": "ral_text_scan_filter_host on the text in page-locked memory (64 MiB pieces copied in while "
                   "the pieces before them are scanned), kept columns copied back"}


def fused_project_setup(n, device):
    import torch
    import ralgpu as R
    from ralgpu import workloads as W
    spec = W.fused_project_program()
    cols = []
    for t, data, valid, nulls in W.fused_project_device(n, device=device):
        cols.append(R.Column(data, valid, t, size=n, null_count=nulls))
    outs = [R.Column.empty(t, n, device=device) for t in spec.output_dtypes]
    bytes_per_row_in = sum(R.dtypes.WIDTH[t] for t in spec.input_dtypes) + len(spec.input_dtypes) / 8
    bytes_per_row_out = sum(R.dtypes.WIDTH[t] for t in spec.output_dtypes) + len(spec.output_dtypes) / 8
    alg_bytes = n * (bytes_per_row_in + bytes_per_row_out)

    def step(stream):
        R.perform_operation_async(outs, cols, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops,
                                  spec.lscalars, spec.rscalars, stream=stream)

    return dict(step=step, alg_bytes=alg_bytes, cols=cols, outs=outs, spec=spec)


def fused_project_e2e(ctx, steps, device):
    """C ABI with host buffers: ral_perform_operation_host over page-locked host columns.  Every
    step copies every input (data + mask) to the device and every output back, in row chunks whose
    copies overlap the kernels; timed by the host clock around the synchronous calls."""
    import torch
    import ralgpu as R
    spec = ctx["spec"]
    n = ctx["cols"][0].size
    host_in = [R.Column(c.data.cpu().pin_memory(), c.valid.cpu().pin_memory(), c.dtype, size=n,
                        null_count=c.null_count) for c in ctx["cols"]]
    host_out = [R.Column(torch.empty_like(o.data, device="cpu").pin_memory(),
                         torch.empty_like(o.valid, device="cpu").pin_memory(), o.dtype, size=n) for o in ctx["outs"]]
    h2d = sum(n * R.dtypes.WIDTH[c.dtype] + (n + 7) // 8 for c in host_in)
    d2h = sum(n * R.dtypes.WIDTH[c.dtype] + (n + 7) // 8 for c in host_out)

    def one():
        R.perform_operation_host(host_out, host_in, spec.left, spec.right, spec.outputs, spec.final, spec.ops,
                                 spec.uops, spec.lscalars, spec.rscalars)

    one()
    one()
    times = []
    for _ in range(max(steps, 5)):
        t0 = time.perf_counter()
        one()
        times.append((time.perf_counter() - t0) * 1e3)
    ms = statistics.median(times)
    return {"value": n / (ms / 1e3), "unit": "rows/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": ms, "timing": f"median of {len(times)} calls after 2 warm-up calls",
            "api": "ral_perform_operation_host (row chunks on three streams)"}


def _colarray(cols):
    import ctypes
    from ralgpu.column import GdfColumn
    structs = [c.to_c() for c in cols]
    arr = (ctypes.POINTER(GdfColumn) * len(structs))()
    for i, st in enumerate(structs):
        arr[i] = ctypes.pointer(st)
    return arr, structs


def filter_setup(workload, n, selectivity, device, null_rate=None):
    """plain_vm (fused filter + project) or filter_gather (fused filter over 6 columns)."""
    import ctypes
    import torch
    import ralgpu as R
    from ralgpu import workloads as W
    L = R.lib()
    if workload == "filter_project":
        frame = []
        for t, data, valid, nulls in W.fused_project_device(n, device=device):
            frame.append(R.Column(data, valid, t, size=n, null_count=nulls))
        fq, pq = W.filter_project_filter(selectivity), W.FILTER_PROJECT_PROJECT
        types, evald = R.project_output_types([c.dtype for c in frame], pq)
        outs = [R.Column.empty(t, n) for t in types]
        in_b = [R.dtypes.WIDTH[c.dtype] + 1 / 8 for c in frame]   # every column (+ mask) is read
        out_b = sum(R.dtypes.WIDTH[t] + 1 / 8 for t in types)
        pred_cols = {4}                               # k < T
    elif workload == "plain_vm":
        spec = W.plain_vm_host(n)
        frame = [R.Column.from_numpy(v, t, m) for t, v, m in spec]
        fq, pq = W.PLAIN_VM_FILTER, W.PLAIN_VM_PROJECT
        types, evald = R.project_output_types([c.dtype for c in frame], pq)
        outs = [R.Column.empty(t, n) for t in types]
        in_b = [8 + 0, 8 + 1 / 8, 4, 4]          # c0, c1 (+mask), c2, c3 read by the predicate / projection
        out_b = 8 + 1 / 8
        pred_cols = {0, 1, 2, 3}
    else:
        frame = []
        for t, data, valid, nulls in W.filter_gather_device(n, device=device, null_rate=null_rate):
            frame.append(R.Column(data, valid, t, size=n, null_count=nulls))
        fq, pq = W.filter_gather_query(selectivity), None
        outs = [R.Column.empty(c.dtype, n, with_valid=c.valid is not None) for c in frame]
        in_b = [R.dtypes.WIDTH[c.dtype] for c in frame]
        out_b = sum(in_b)
        pred_cols = {0}                               # <($0, T)
    fa, fs = _colarray(frame)
    oa, os_ = _colarray(outs)
    nout = ctypes.c_int32(0)

    def step(stream):
        if pq is None:
            rc = L.ral_process_filter(fa, len(frame), fq.encode(), oa, ctypes.byref(nout))
        else:
            rc = L.ral_filter_project(fa, len(frame), fq.encode(), pq.encode(), oa, len(outs), ctypes.byref(nout))
        if rc:
            raise RuntimeError(L.ral_last_error().decode())

    def alg_bytes():
        k = nout.value
        return n * sum(in_b) + k * out_b + 8

    def touched_bytes():
        """The bytes the kernel reaches at this selectivity: the predicate's columns whole, every
        other column's 32-byte sectors that hold a kept row (kept rows independent with
        probability s: a sector of r rows is touched with probability 1 - (1 - s)^r), the masks'
        sectors alike, and the kept rows written."""
        k = nout.value
        sel = k / max(n, 1)
        total = k * out_b
        for i, c in enumerate(frame):
            w = R.dtypes.WIDTH[c.dtype]
            if i in pred_cols:
                total += n * w + (n / 8 if c.valid is not None else 0)
                continue
            total += n * w * (1 - (1 - sel) ** (32 / w))
            if c.valid is not None:
                total += n / 8 * (1 - (1 - sel) ** 256)
        return total

    return dict(step=step, alg_bytes_fn=alg_bytes, touched_bytes_fn=touched_bytes, nout=nout, cols=frame, outs=outs, out_structs=os_, fq=fq, pq=pq)


def gather_setup(n, pattern, device, null_rate=0.05):
    """Every column of the six-column frame of filter_gather (int32, int64, float32, float64, date32,
    bool8; 5% nulls) gathered by one int32 index column: a permutation (order-by), random indices
    with repetition (join) or sorted random indices (the kept rows of a filter)."""
    import ctypes
    import torch
    import ralgpu as R
    from ralgpu import dtypes as D
    from ralgpu import workloads as W
    L = R.lib()
    frame = [R.Column(v, m, t, n, nn) for t, v, m, nn in W.filter_gather_device(n, device=device, null_rate=null_rate)]
    g = torch.Generator(device=device)
    g.manual_seed(W.SEED + 1)
    if pattern == "permutation":
        idx = torch.randperm(n, generator=g, device=device, dtype=torch.int32)
    else:
        idx = torch.randint(0, n, (n,), generator=g, device=device, dtype=torch.int32)
        if pattern == "sorted":
            idx = torch.sort(idx).values
    icol = R.Column(idx, None, D.GDF_INT32, n)
    outs = [R.Column.empty(c.dtype, n, with_valid=c.valid is not None, device=device) for c in frame]
    fa, fs = _colarray(frame)
    oa, os_ = _colarray(outs)
    ic = icol.to_c()

    def step(stream):
        rc = L.ral_materialize_columns(ctypes.cast(fa, ctypes.c_void_p), ctypes.cast(oa, ctypes.c_void_p),
                                       len(frame), ctypes.byref(ic))
        if rc:
            raise RuntimeError(L.ral_last_error().decode())

    def per_column(stream):
        for c, o in zip(fs, os_):
            rc = L.ral_materialize_column(ctypes.byref(c), ctypes.byref(o), ctypes.byref(ic))
            if rc:
                raise RuntimeError(L.ral_last_error().decode())

    widths = [D.WIDTH[c.dtype] for c in frame]
    masked = [c.valid is not None for c in frame]
    # algorithmic: the index, one element read and one written per column, masks read and written
    alg = n * (4 + sum(2 * w for w in widths) + sum(2 / 8 for m in masked if m))
    return dict(step=step, per_column=per_column, alg_bytes=alg, cols=frame, outs=outs, idx=icol,
                out_structs=os_, pattern=pattern)


def gather_parity(ctx):
    """Every output row of every column against the oracle's materialize_column, in chunks of
    output rows on all host threads."""
    import concurrent.futures as cf
    import numpy as np
    import oracle as O
    t0 = time.perf_counter()
    threads = os.cpu_count() or 1
    n = ctx["idx"].size
    idx = ctx["idx"].data[:n].cpu().numpy()
    stats = {"valid": 0, "data": 0, "null_count": 0}
    chunk = PARITY_CHUNK
    for c, (col, out, st) in enumerate(zip(ctx["cols"], ctx["outs"], ctx["out_structs"])):
        host = _oracle_chunk([col], 0, col.size)[0]

        def one(s):
            e = min(n, s + chunk)
            exp = O.materialize_column(host, idx[s:e])
            local = {"valid": 0, "data": 0}
            _compare(out, s, e, exp, local)
            return local, (exp.null_count if exp.valid is not None else 0)

        nulls = 0
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            for local, nc in ex.map(one, range(0, n, chunk)):
                stats["valid"] += local["valid"]
                stats["data"] += local["data"]
                nulls += nc
        stats["null_count"] += int(st.null_count != nulls)
        del host
    return {"rows": n, "columns": len(ctx["cols"]), "mismatches": sum(stats.values()), "detail": stats,
            "checked": "every output row of every column, bit for bit: data of valid rows, validity bits, null counts",
            "oracle_threads": threads, "seconds": round(time.perf_counter() - t0, 2)}


def cpu_gather(rows: int, threads: int):
    """The oracle's materialize_column over every column of the frame, output chunks on threads."""
    import concurrent.futures as cf
    import numpy as np
    import oracle as O
    from ralgpu import workloads as W
    frame = [O.make_column(v, t, m) for t, v, m in W.filter_gather_host(rows, seed=99, null_rate=0.05)]
    idx = np.random.default_rng(5).permutation(rows).astype(np.int32)
    step = max(1, (rows + threads - 1) // threads)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda s: [O.materialize_column(c, idx[s:s + step]) for c in frame], range(0, rows, step)))
    return time.perf_counter() - t0


def filter_e2e(ctx, steps):
    """C ABI with host buffers: ral_filter_project_host over page-locked host columns into
    page-locked host outputs -- row chunks streamed through the GPU on three streams, each chunk's
    kept rows copied back to their place as soon as its count is known."""
    import torch
    import ralgpu as R
    from ralgpu import dtypes as D
    n = ctx["cols"][0].size
    host_in = [R.Column(c.data.cpu().pin_memory(), None if c.valid is None else c.valid.cpu().pin_memory(),
                        c.dtype, n, c.null_count) for c in ctx["cols"]]
    host_out = [R.Column(torch.empty(max(n, 1), dtype=D.torch_dtype(o.dtype)).pin_memory(),
                         None if o.valid is None else torch.empty(R.valid_alloc_size(n), dtype=torch.uint8).pin_memory(),
                         o.dtype, n) for o in ctx["outs"]]

    def one():
        return R.filter_project_host(host_in, ctx["fq"], ctx["pq"], host_out)

    one()
    one()
    times = []
    k = 0
    for _ in range(max(steps, 5)):
        t0 = time.perf_counter()
        k = one()
        times.append((time.perf_counter() - t0) * 1e3)
    ms = statistics.median(times)
    h2d = sum(c.data.numel() * c.data.element_size() + (0 if c.valid is None else (n + 7) // 8) for c in host_in)
    d2h = sum(k * o.data.element_size() + (0 if o.valid is None else (k + 7) // 8) for o in host_out)
    return {"value": n / (ms / 1e3), "unit": "rows/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": ms, "timing": f"median of {len(times)} calls after 2 warm-up calls",
            "api": "ral_filter_project_host (row chunks streamed on three streams)"}


# ---- full-size parity: the oracle as the checker, outside every timed region ----------------

PARITY_CHUNK = 1 << 24   # input rows per oracle chunk (a multiple of 64: chunk masks start on a byte)


def _bits_np(valid, s, e):
    """Validity bits [s, e) of a packed device mask as a numpy bool array."""
    import numpy as np
    if valid is None:
        return np.ones(e - s, dtype=bool)
    raw = valid[s // 8:(e + 7) // 8].cpu().numpy()
    return np.unpackbits(raw, bitorder="little")[s % 8:s % 8 + (e - s)].astype(bool)


def _oracle_chunk(cols, s, e):
    """Oracle columns holding rows [s, e) of device columns; each keeps its whole column's null count,
    which the interpreter's validity pass reads (null_count == 0 means all-valid)."""
    import numpy as np
    import oracle as O
    out = []
    for c in cols:
        data = np.ascontiguousarray(c.data[s:e].cpu().numpy())
        if c.valid is None:
            out.append(O.OColumn(data, None, c.dtype, 0))
        else:
            out.append(O.make_column(data, c.dtype, _bits_np(c.valid, s, e), null_count=c.null_count))
    return out


def _compare(gpu_col, g0, g1, oc, stats):
    """Rows [g0, g1) of a device output against an oracle column: validity bits, and the data bits
    of every valid row (data under a null is unspecified)."""
    import numpy as np
    gv = _bits_np(gpu_col.valid, g0, g1)
    ov = oc.valid_bools()[:g1 - g0] if oc.valid is not None else np.ones(g1 - g0, dtype=bool)
    if gpu_col.valid is not None or oc.valid is not None:
        stats["valid"] += int((gv != ov).sum())
    m = gv & ov
    gd = gpu_col.data[g0:g1].cpu().numpy()
    od = oc.data[:g1 - g0]
    u = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[gd.dtype.itemsize]
    stats["data"] += int((gd.view(u)[m] != od.astype(gd.dtype, copy=False).view(u)[m]).sum())


def parity_check(workload, ctx, selectivity):
    """Runs the oracle over every input row of the last timed step (in chunks of PARITY_CHUNK rows on
    all host threads) and compares every output row bit for bit: data of valid rows, validity bits,
    null counts, the kept row count and row order."""
    import oracle as O
    from ralgpu import workloads as W
    t0 = time.perf_counter()
    threads = os.cpu_count() or 1
    cols, outs = ctx["cols"], ctx["outs"]
    n = cols[0].size
    stats = {"valid": 0, "data": 0, "rows_out": 0, "null_count": 0}
    kept = 0
    nulls = [0] * len(outs)
    for s in range(0, n, PARITY_CHUNK):
        e = min(n, s + PARITY_CHUNK)
        chunk = _oracle_chunk(cols, s, e)
        if workload == "fused_project":
            spec = ctx["spec"]
            from oracle import frontend as fe
            exp = [O.alloc_column(t, e - s) for t in spec.output_dtypes]
            O.perform_operation(exp, chunk, spec.left, spec.right, spec.outputs, spec.final, spec.ops, spec.uops,
                                [fe.Scalar(*x) for x in spec.lscalars], [fe.Scalar(*x) for x in spec.rscalars],
                                nthreads=threads)
            g0, k = s, e - s
        else:
            f = O.process_filter(chunk, ctx["fq"], nthreads=threads)
            exp = f if ctx["pq"] is None else O.execute_project_plan(f, ctx["pq"], nthreads=threads)
            k = exp[0].size
            g0 = kept
            for i, oc in enumerate(exp):
                O.update_null_count(oc)
                nulls[i] += oc.null_count
        for gcol, oc in zip(outs, exp):
            if k:
                _compare(gcol, g0, g0 + k, oc, stats)
        kept += k
    out = {"rows": n, "chunks": (n + PARITY_CHUNK - 1) // PARITY_CHUNK, "oracle_threads": threads}
    if "nout" in ctx:
        got = ctx["nout"].value
        stats["rows_out"] = abs(got - kept)
        out["rows_out"] = got
        for i, st in enumerate(ctx["out_structs"]):
            stats["null_count"] += int(st.null_count != nulls[i])
    out["mismatches"] = sum(stats.values())
    out["detail"] = stats
    out["checked"] = ("every output row, bit for bit: data of valid rows, validity bits"
                      + (", null counts, kept row count and row order" if "nout" in ctx else ""))
    out["seconds"] = round(time.perf_counter() - t0, 2)
    return out


_LINK = None


def host_link_peak(nbytes=1 << 30, reps=5):
    """Pinned host <-> device copy bandwidth with plain cudaMemcpyAsync (torch copies): H2D alone,
    D2H alone, and both directions at once on two streams (GB/s, best of reps).  Measured once."""
    global _LINK
    if _LINK is not None:
        return _LINK
    import torch
    h_in = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    h_out = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d_a = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d_b = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(fn):
        best = 1e30
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    def both():
        with torch.cuda.stream(s1):
            d_a.copy_(h_in, non_blocking=True)
        with torch.cuda.stream(s2):
            h_out.copy_(d_b, non_blocking=True)

    h2d = nbytes / timed(lambda: d_a.copy_(h_in, non_blocking=True)) / 1e9
    d2h = nbytes / timed(lambda: h_out.copy_(d_b, non_blocking=True)) / 1e9
    bi = 2 * nbytes / timed(both) / 1e9
    _LINK = {"h2d_gbs": h2d, "d2h_gbs": d2h, "both_gbs": bi,
             "how": f"pinned {nbytes >> 20} MiB cudaMemcpyAsync, best of {reps}; both = H2D and D2H at once"}
    del h_in, h_out, d_a, d_b
    return _LINK


def aggregate_oracle_chunked(cols, query):
    """The oracle's process_aggregate over device columns of any size: rows in chunks of
    PARITY_CHUNK on all host threads, partial results combined (integer sums modulo 2^64, exact float
    sums of the partial sums, MIN / MAX, counts; AVG as the combined sum over the combined count)."""
    import math
    import numpy as np
    import oracle as O
    from oracle import frontend as fe
    threads = os.cpu_count() or 1
    n = cols[0].size
    _, aggs = fe.parse_aggregate(query)
    # per chunk: AVG reduced as SUM; its count is the evaluated row count or the bare valid count
    chunk_q = query.replace("=[AVG(", "=[SUM(")
    parts = [[] for _ in aggs]
    counts = [0] * len(aggs)
    for s0 in range(0, n, PARITY_CHUNK):
        e0 = min(n, s0 + PARITY_CHUNK)
        frame = []
        for c in cols:
            data = np.ascontiguousarray(c.data[s0:e0].cpu().numpy())
            frame.append(O.OColumn(data, None, c.dtype, 0) if c.valid is None
                         else O.make_column(data, c.dtype, _bits_np(c.valid, s0, e0)))
        res = O.process_aggregate(frame, chunk_q, nthreads=threads)
        for i, ((name, op, expr), r) in enumerate(zip(aggs, res)):
            parts[i].append(r)
            if op == fe.GDF_AVG:
                col = None if fe.contains_evaluation(expr) else frame[fe.get_index(expr)]
                counts[i] += (e0 - s0) if col is None else col.size - col.null_count
    out = []
    for i, (name, op, expr) in enumerate(aggs):
        ps = parts[i]
        valid = [p for p in ps if p.is_valid]
        t = ps[0].dtype if ps else fe.GDF_INT64
        if op == fe.GDF_COUNT:
            out.append(O.AggResult(fe.GDF_INT64, True, sum(p.value for p in ps)))
        elif not valid:
            out.append(O.AggResult(fe.GDF_FLOAT64 if op == fe.GDF_AVG else t, False))
        elif op in (fe.GDF_MIN, fe.GDF_MAX):
            v = min(p.value for p in valid) if op == fe.GDF_MIN else max(p.value for p in valid)
            out.append(O.AggResult(t, True, v))
        else:
            bound = sum(p.float_sum_bound for p in valid)
            if isinstance(valid[0].value, float):
                total = math.fsum(p.value for p in valid)
            else:
                total = int(np.array([p.value for p in valid], dtype=np.int64).astype(np.uint64)
                            .sum(dtype=np.uint64).astype(np.int64))
            if op == fe.GDF_SUM:
                out.append(O.AggResult(t, True, total, bound))
            else:
                out.append(O.AggResult(fe.GDF_FLOAT64, True, float(total) / counts[i], bound / counts[i]))
    return out


def measure_workload(args, workload, n, selectivity, device, world, sampler, e2e=True, cpu=True, parity=True,
                     cpu_budget_s=12.0):
    """One workload: warm-up, the timed steps (CUDA events on the launching stream, max over ranks),
    the roofline of its kernel, and on rank 0 the e2e, CPU baseline and full-size parity legs."""
    import torch
    import ralgpu as R
    rank = int(os.environ.get("RANK", "0"))
    if workload == "fused_project":
        ctx = fused_project_setup(n, device)
    elif workload == "scan_filter":
        ctx = scan_filter_setup(n, device)
    elif workload in PARQUET_WORKLOADS:
        ctx = parquet_filter_setup(n, device, dictionary=workload == "parquet_dict_filter")
    elif workload == "gather":
        ctx = gather_setup(n, selectivity, device)
    else:
        ctx = filter_setup(workload, n, selectivity, device)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        ctx["step"](stream)
    torch.cuda.synchronize()
    barrier(world)
    launches0 = R.kernel_launches()
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    w0 = time.monotonic()
    if workload == "plain_vm":
        # a per-call latency: the K calls back to back with only the two outer events (a pair of
        # event records per call would add their host cost to every call), then the same calls
        # again with per-call events for the kernel's own duration
        t_start.record()
        for _ in events:
            ctx["step"](stream)
        t_end.record()
        torch.cuda.synchronize()
        for s, e in events:
            s.record()
            ctx["step"](stream)
            e.record()
    else:
        t_start.record()
        for s, e in events:
            s.record()
            ctx["step"](stream)
            e.record()
        t_end.record()
    torch.cuda.synchronize()
    w1 = time.monotonic()
    launches = R.kernel_launches() - launches0
    if workload == "plain_vm":
        launches //= 2
    barrier(world)
    total_ms = max_over_ranks(world, t_start.elapsed_time(t_end))
    kernel_ms = statistics.mean(s.elapsed_time(e) for s, e in events)
    ms_per_step = total_ms / args.steps
    peak, peak_kind = load_peaks()
    alg = ctx["alg_bytes"] if "alg_bytes" in ctx else ctx["alg_bytes_fn"]()
    achieved = alg / (kernel_ms / 1e3) / 1e9
    traffic_key = workload if workload not in ("filter_gather", "filter_project", "gather") else f"{workload}_{selectivity}"
    out = {
        "workload": workload, "value": job_rate(world, n, ms_per_step), "unit": "rows/s", "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step,
        "config": workload_config(workload, n, selectivity, world),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                     "frac_of_8tbs": achieved / 8000.0, "traffic": load_traffic(traffic_key),
                     "algorithmic_bytes_per_launch": alg, "kernel_ms": kernel_ms},
        "gpu_launches": int(launches),
        "clocks": sampler.window(w0, w1),
    }
    if "nout" in ctx:
        out["rows_out"] = ctx["nout"].value
    if "touched_bytes_fn" in ctx:
        # below s = 50% the kernel reads the non-predicate columns only around kept rows: the
        # fraction against the bytes it can reach stays below 1 where the full-read one would not
        touched = ctx["touched_bytes_fn"]()
        out["roofline"]["touched_model_bytes_per_launch"] = touched
        out["roofline"]["touched_model_gbs"] = touched / (kernel_ms / 1e3) / 1e9
        out["roofline"]["touched_model_frac"] = out["roofline"]["touched_model_gbs"] / peak
    if workload == "plain_vm":
        # where a small synchronous call's time goes: the same calls again with the library's
        # per-call timing on (host preparation, enqueue, wait, kernel device time)
        R.call_timing(enable=True, reset=True)
        for _ in range(max(20, args.steps)):
            ctx["step"](stream)
        torch.cuda.synchronize()
        out["per_call_breakdown_us"] = R.call_timing(enable=False, reset=True)
        out["per_call_breakdown_us"]["call_us"] = ms_per_step * 1e3
        # the roofline of the kernel itself: its device time inside the call, not the call's
        kus = out["per_call_breakdown_us"]["kernel_device_us"]
        if kus > 0:
            rl = out["roofline"]
            rl["kernel_ms"] = kus / 1e3
            rl["achieved"] = alg / (kus / 1e6) / 1e9
            rl["frac"] = rl["achieved"] / peak
            rl["frac_of_8tbs"] = rl["achieved"] / 8000.0
            rl["kernel_time"] = "CUDA events around the filter kernel launch inside the call (library call timing)"
    if workload == "gather":
        # the same gather as one ral_materialize_column call per column (the reference's loop shape)
        for _ in range(2):
            ctx["per_column"](stream)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
        for a, b in ev:
            a.record()
            ctx["per_column"](stream)
            b.record()
        torch.cuda.synchronize()
        pc = statistics.mean(a.elapsed_time(b) for a, b in ev)
        out["per_column_calls"] = {"ms_per_step": pc, "value": n / (pc / 1e3), "calls": len(ctx["cols"]),
                                   "speedup_of_fused": pc / ms_per_step,
                                   "api": "ral_materialize_column once per column, index read each time"}
        # a random gather reads one 32-byte sector per element and mask word (inputs exceed L2)
        if ctx["pattern"] != "sorted":
            touched = n * (4 + sum(32 + w for w in (R.dtypes.WIDTH[c.dtype] for c in ctx["cols"]))
                           + sum(32 + 1 / 8 for c in ctx["cols"] if c.valid is not None))
            out["roofline"]["sector_model_bytes_per_launch"] = touched
            out["roofline"]["sector_model_gbs"] = touched / (kernel_ms / 1e3) / 1e9
    if rank == 0:
        if e2e and not args.skip_e2e and workload != "gather":
            if workload == "fused_project":
                out["e2e"] = fused_project_e2e(ctx, max(2, min(args.steps, 3)), device)
            elif workload == "scan_filter":
                out["e2e"] = scan_filter_e2e(ctx, max(2, min(args.steps, 3)))
            elif workload in PARQUET_WORKLOADS:
                # the call itself starts from host memory: its step time is the end-to-end time
                out["e2e"] = {"value": out["value"], "unit": "rows/s", "h2d_bytes_per_step": int(ctx["chunk_bytes"]),
                              "d2h_bytes_per_step": 0, "ms_per_step": out["ms_per_step"],
                              "api": "ral_parquet_scan_filter on the file in page-locked host memory (kept rows stay "
                                     "on the device)"}
            else:
                out["e2e"] = filter_e2e(ctx, max(2, min(args.steps, 3)))
            link = host_link_peak()
            bi, bo = out["e2e"]["h2d_bytes_per_step"], out["e2e"]["d2h_bytes_per_step"]
            out["e2e"]["host_link"] = dict(link, e2e_gbs=(bi + bo) / (out["e2e"]["ms_per_step"] / 1e3) / 1e9)
            # the copies alone at the measured rates: each direction at its own rate, both at once
            # no faster than the two-stream figure
            floor_ms = max(bi / (link["h2d_gbs"] * 1e9), bo / (link["d2h_gbs"] * 1e9), (bi + bo) / (link["both_gbs"] * 1e9)) * 1e3
            out["e2e"]["host_link"]["copy_floor_ms"] = floor_ms
            out["e2e"]["host_link"]["frac_of_link"] = floor_ms / out["e2e"]["ms_per_step"]
        # the device outputs (the e2e leg rewrote them with the same bits) against the oracle
        if parity and not args.skip_parity:
            out["parity"] = (gather_parity(ctx) if workload == "gather" else
                             scan_filter_parity(ctx) if workload in ("scan_filter",) + PARQUET_WORKLOADS else
                             parity_check(workload, ctx, selectivity))
        if cpu and not args.skip_cpu and workload not in PARQUET_WORKLOADS:
            out["cpu_baseline"] = cpu_baseline(workload, n, selectivity, budget_s=cpu_budget_s,
                                               single_budget_s=cpu_budget_s / 3)
        if cpu and not args.skip_cpu and workload in PARQUET_WORKLOADS:
            out["cpu_baseline"] = cpu_parquet(ctx, budget_s=min(cpu_budget_s, 6.0))
    del ctx
    torch.cuda.empty_cache()
    return out


# Workloads measured beside the default one in the same run: the 200M-row fused filter + project at
# s = 0.5 (the target kernel) and the 500M-row filter + gather of six columns at s = 0.5.
EXTRA_WORKLOADS = [("filter_project", 0.5), ("filter_gather", 0.5), ("gather", "permutation"), ("scan_filter", None),
                   ("parquet_filter", None), ("parquet_dict_filter", None)]


def run_ours(args):
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    n = args.rows or DEFAULT_ROWS[args.workload]
    sampler = ClockSampler(local)
    sampler.start()
    sel = args.pattern if args.workload == "gather" else args.selectivity
    main = measure_workload(args, args.workload, n, sel, device, world, sampler)
    extra = {}
    if args.workload == "fused_project" and not args.rows and not args.no_extra:
        for wl, sel in EXTRA_WORKLOADS:
            key = wl if sel is None else f"{wl}_{sel}" if isinstance(sel, str) else f"{wl}_s{sel}"
            extra[key] = measure_workload(args, wl, DEFAULT_ROWS[wl], sel, device, world, sampler, cpu_budget_s=6.0)
    sampler.stop()
    out = {
        "metric": METRIC, "value": main["value"], "unit": "rows/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"fused_project": "f64+int64", "filter_project": "f64+int64", "plain_vm": "f64+int64",
                  "filter_gather": "int32/int64/f32/f64/date32/bool8 gather",
                  "gather": "int32/int64/f32/f64/date32/bool8 gather",
                  "scan_filter": "u8 text -> int32/f64/date64",
                  "parquet_filter": "Parquet pages -> int32/f64/date64",
                  "parquet_dict_filter": "Parquet pages -> int32/f64/date64"}[args.workload],
        "data": "synthetic (seeded, generated on the GPU)",
        "config": main["config"],
        "hbm_gbs": main["roofline"]["achieved"],
        "roofline": main["roofline"],
        "gpu_launches": main["gpu_launches"] + sum(b["gpu_launches"] for b in extra.values()),
        "gpu_launches_main": main["gpu_launches"],
        "clocks": main["clocks"],
    }
    for k in ("rows_out", "parity", "e2e", "cpu_baseline", "per_call_breakdown_us", "per_column_calls"):
        if k in main:
            out[k] = main[k]
    if extra:
        out["extra_workloads"] = extra
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def batched_config(args, world=1):
    """`config` of the batched workload (the same dict on both arms)."""
    from ralgpu import workloads as W
    mix = W.batched_mix(args.programs, seed=args.seed)
    rows = sum(min(t.rows, args.max_rows) if args.max_rows else t.rows for t in mix)
    return {"workload": "batched", "programs": len(mix), "rows_total": int(rows), "ops": "4-48 per program",
            "rows_per_table": "log-uniform [1e3, 5e7]", "columns": "2-8 of int32/int64/f32/f64, 0-20% nulls",
            "seed": args.seed, "parallelism": f"replicas x{world}", "max_rows": args.max_rows or None,
            "l2": "inputs of the whole batch (tens of GB) exceed L2; no flush"}


def served_config(args, world=1):
    """`config` of the served workload (the same dict on both arms)."""
    from ralgpu import workloads as W
    tabs = W.served_tables(args.tables, seed=args.seed, max_rows=args.max_rows or 1e8)
    n_rate = max(50, args.requests // 5)
    return {"workload": "served", "tables": len(tabs), "rows_resident": int(sum(t.rows for t in tabs)),
            "queries": args.queries, "ops": "4-32 per request (filter + project)", "nulls": "5% per column",
            "requests": int(n_rate * 5), "arrivals": "Poisson, 5 rates",
            "budget_gb": args.budget_gb, "max_waves": args.waves, "wave_rows": args.wave_rows or "default",
            "parallelism": f"replicas x{world}",
            "l2": "tables of up to 1e8 rows exceed L2; no flush"}


def batched_setup(n_programs, seed, device, max_rows=0):
    """Device tables, outputs and plans of the batched mix (tables capped at max_rows when set,
    for small profiling captures)."""
    import torch
    import ralgpu as R
    from ralgpu import dtypes as D
    from ralgpu import workloads as W
    mix = W.batched_mix(n_programs, seed=seed)
    progs = []
    alg = 0
    for t in mix:
        if max_rows:
            t.rows = min(t.rows, max_rows)
        pp = R.parse_project_plan(t.dtypes, t.project)
        cols = W.batched_table_device(t, device)
        ins = [R.Column(cols[c][1], cols[c][2], cols[c][0], t.rows, cols[c][3]) for c in pp["input_columns"]]
        outs = [R.Column.empty(dt, t.rows, with_valid=True, device=device) for dt in pp["evaluated_dtypes"]]
        args = (pp["left"], pp["right"], pp["outputs"], pp["final_output_positions"], pp["operators"],
                pp["unary_operators"], pp["left_scalars"], pp["right_scalars"])
        # algorithmic bytes: every input column read once (data + mask), every output written once
        b = sum(t.rows * D.WIDTH[c.dtype] + (0 if c.valid is None else (t.rows + 7) // 8) for c in ins)
        b += sum(t.rows * D.WIDTH[dt] + (t.rows + 7) // 8 for dt in pp["evaluated_dtypes"])
        alg += b
        progs.append(dict(t=t, pp=pp, ins=ins, outs=outs, args=args, rows=t.rows))
    torch.cuda.synchronize()
    return progs, alg


def batched_capped(R, progs, cap, stream, plain_steps):
    """Batched vs plain calls for the same programs over the first `cap` rows of every table."""
    import torch
    views = []
    for p in progs:
        n = min(p["rows"], cap)
        ins = [R.Column(c.data[:n], c.valid, c.dtype, n, c.null_count) for c in p["ins"]]
        outs = [R.Column(c.data[:n], c.valid, c.dtype, n) for c in p["outs"]]
        views.append((ins, outs, p["args"], n))
    rows = sum(v[3] for v in views)
    b = R.Batch()
    for ins, outs, a, n in views:
        b.add(outs, ins, *a)
    b.prepare()
    for _ in range(3):
        b.run(stream)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
    for s_, e_ in ev:
        s_.record(stream)
        b.run(stream)
        e_.record(stream)
    torch.cuda.synchronize()
    bms = statistics.mean(s_.elapsed_time(e_) for s_, e_ in ev)
    b.close()
    for ins, outs, a, n in views:
        R.perform_operation(outs, ins, *a)
    torch.cuda.synchronize()
    times = []
    for _ in range(plain_steps):
        t0 = time.perf_counter()
        for ins, outs, a, n in views:
            R.perform_operation(outs, ins, *a)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    pms = statistics.median(times) * 1e3
    return {"cap_rows": cap, "rows": rows, "batched_ms": bms, "plain_ms": pms,
            "batched_rows_per_s": rows / (bms / 1e3), "plain_rows_per_s": rows / (pms / 1e3),
            "speedup_vs_plain": pms / bms}


def batched_floor_block(args, clocks, ms_per_step, plain):
    """The floor of the default mix from the committed per-program counters, at the clock measured
    during the timed region; None for another mix."""
    p = os.path.join(ROOT, "profiles", "batch_mix_fp64.json")
    if not os.path.exists(p) or args.max_rows or args.programs != 256 or args.seed != 20261203:
        return None
    table = json.load(open(p))
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    peak, _ = load_peaks()
    f = batch_floor(table, float(mhz), peak)
    f["batched_frac_of_floor"] = f["floor_ms"] / ms_per_step
    if plain:
        f["plain_frac_of_floor"] = f["per_program_floor_ms"] / plain["ms_per_step"]
        f["max_speedup_over_plain"] = plain["ms_per_step"] / f["floor_ms"]
    return f


def run_batched(args):
    import concurrent.futures as cf
    import torch
    import ralgpu as R
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    t0 = time.perf_counter()
    progs, alg = batched_setup(args.programs, args.seed, device, args.max_rows)
    rows = sum(p["rows"] for p in progs)
    gen_s = time.perf_counter() - t0
    # autotune: one program per tuning key (dtype mix x program length), timed as a batch item
    t0 = time.perf_counter()
    tuned = {}
    if not args.no_autotune:
        from collections import OrderedDict
        keys = OrderedDict()
        for p in progs:
            k = R.batch_tune_key(p["outs"], p["ins"], *p["args"])
            if k not in keys or p["rows"] > keys[k]["rows"]:
                keys[k] = p
        for k, p in keys.items():
            J, U, soft, ms = R.autotune_program(p["outs"], p["ins"], *p["args"])
            tuned[k] = [J, U, int(soft), round(ms, 4)]
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = R.Batch()
    for p in progs:
        b.add(p["outs"], p["ins"], *p["args"])
    b.prepare()
    prep_s = time.perf_counter() - t0
    info = b.info()
    stream = torch.cuda.current_stream()
    sampler = ClockSampler(local)
    sampler.start()
    for _ in range(args.warmup):
        b.run(stream)
    torch.cuda.synchronize()
    barrier(world)
    launches0 = R.kernel_launches()
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sampler.mark_start()
    for s_, e_ in events:
        s_.record(stream)
        b.run(stream)
        e_.record(stream)
    torch.cuda.synchronize()
    sampler.mark_end()
    launches = R.kernel_launches() - launches0
    clocks = sampler.stop()
    step_ms = [s_.elapsed_time(e_) for s_, e_ in events]
    ms_per_step = max_over_ranks(world, statistics.mean(step_ms))
    value = job_rate(world, rows, ms_per_step)

    # the same programs as plain per-call launches: one synchronous ral_perform_operation each
    plain = None
    if args.plain_steps > 0:
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:   # compile the kernels
            list(ex.map(lambda p: R.perform_operation(p["outs"], p["ins"], *p["args"]), progs))
        torch.cuda.synchronize()
        plain_compile_s = time.perf_counter() - t0
        for p in progs:
            R.perform_operation(p["outs"], p["ins"], *p["args"])
        torch.cuda.synchronize()
        plain_times = []
        for _ in range(args.plain_steps):
            t0 = time.perf_counter()
            for p in progs:
                R.perform_operation(p["outs"], p["ins"], *p["args"])
            torch.cuda.synchronize()
            plain_times.append(time.perf_counter() - t0)
        plain_s = statistics.median(plain_times)
        plain = {"value": world * rows / plain_s, "unit": "rows/s", "ms_per_step": plain_s * 1e3,
                 "calls_per_step": len(progs), "steps": args.plain_steps,
                 "timing": "host clock around synchronous ral_perform_operation calls, one per program",
                 "first_compile_s": round(plain_compile_s, 2)}

    # the same 256 programs over the first cap rows of each table (views of the same columns):
    # where per-call cost, not the FP64 work of the few largest tables, decides
    capped = None
    if args.plain_steps > 0 and args.capped_rows > 0:
        capped = batched_capped(R, progs, args.capped_rows, stream, args.plain_steps)

    peak, peak_kind = load_peaks()
    achieved = alg / (ms_per_step / 1e3) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32/int64/f32/f64 (VM registers int64/f64)",
        "data": "synthetic (seeded, generated on the GPU)",
        "config": batched_config(args, world),
        "batched": {"launch": "one persistent kernel per step, replayed as a CUDA graph",
                    "kernel": info, "ms_per_step": ms_per_step,
                    "prepare_s": round(prep_s, 2), "autotune_s": round(tune_s, 2), "tuned_keys": len(tuned),
                    "tuned_integer_pipe_keys": sum(v[2] for v in tuned.values()),
                    "generate_s": round(gen_s, 2)},
        "plain_per_call": plain,
        "speedup_vs_plain": value / plain["value"] if plain else None,
        "floor": batched_floor_block(args, clocks, ms_per_step, plain),
        "capped_tables": capped,
        "hbm_gbs": achieved,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                     "traffic": load_traffic("batched"), "algorithmic_bytes_per_launch": alg,
                     "kernel_ms": ms_per_step,
                     "note": "programs with FP64 transcendentals are bound by the FP64 pipe, not HBM"},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "e2e": None,
        "e2e_note": "batched tables are device-resident by design (the served model); host round trips are "
                    "measured on the fused_project and filter workloads",
    }
    if rank == 0:
        if not args.skip_cpu:
            threads = os.cpu_count() or 1
            r, sec = cpu_batched(threads, 64, 200_000, args.seed)
            out["cpu_baseline"] = {"value": r / sec, "unit": "rows/s", "cores": threads, "kind": "port",
                                   "sample": f"first 64 programs of the mix, tables capped at 200000 rows ({r} rows)"}
        print(json.dumps(out), flush=True)
    b.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def _plain_filter_project_call(R, frame, q):
    """A synchronous ral_filter_project over a resident table with preallocated outputs; returns
    a zero-argument callable (the serial plain execution of one request)."""
    import ctypes as C
    from ralgpu.capi import _colarray, lib, _check
    types, evald = R.project_output_types([c.dtype for c in frame], q.project)
    srcs = R.capi._passthrough_sources(frame, q.project)
    n = frame[0].size
    outs = [R.Column.empty(t, n, with_valid=True if e else (srcs[i].valid is not None))
            for i, (t, e) in enumerate(zip(types, evald))]
    fa, fs = _colarray(frame)
    oa, os_ = _colarray(outs)
    fq, pq = q.filter.encode(), q.project.encode()
    n_out = C.c_int32(0)
    keep = (outs, fa, fs, oa, os_)

    def call():
        _check(lib().ral_filter_project(keep[1], len(frame), fq, pq, keep[3], len(keep[0]), C.byref(n_out)))
        return n_out.value
    return call


def run_served(args):
    import numpy as np
    import torch
    import ralgpu as R
    from ralgpu import workloads as W
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    t0 = time.perf_counter()
    tabs = W.served_tables(args.tables, seed=args.seed, max_rows=args.max_rows or 1e8)
    qs = W.served_queries(tabs, args.queries, seed=args.seed)
    frames = []
    for t in tabs:
        cols = W.served_table_device(t, device)
        frames.append([R.Column(v, m, dt, t.rows, nn) for dt, v, m, nn in cols])
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    budget = int(args.budget_gb * (1 << 30))
    srv = R.Server(budget_bytes=budget, max_waves=args.waves, max_wave_requests=1024,
                   wave_rows=args.wave_rows)
    tids = [srv.add_table(f) for f in frames]
    qids = [srv.add_query(tids[q.table], q.filter, q.project) for q in qs]
    t0 = time.perf_counter()
    srv.start()
    start_s = time.perf_counter() - t0
    q_rows = np.array([tabs[q.table].rows for q in qs], dtype=np.float64)

    # serial plain execution: each query's service time as one synchronous ral_filter_project
    calls = [_plain_filter_project_call(R, frames[q.table], q) for q in qs]
    for c in calls:
        c()
    torch.cuda.synchronize()
    service = np.zeros(len(qs))
    for i, c in enumerate(calls):
        ts = []
        for _ in range(3):
            a = time.perf_counter()
            c()
            ts.append(time.perf_counter() - a)
        service[i] = statistics.median(ts)
    del calls
    torch.cuda.empty_cache()

    # warm the served loop, then its capacity: every request of a trace arriving at once
    n_rate = max(50, args.requests // 5)
    wq, wa = W.served_trace(min(500, n_rate), 1e9, len(qs), seed=args.seed + 99)
    srv.run_trace(wq, np.zeros(len(wq)))
    cq, _ = W.served_trace(min(4000, 2 * n_rate), 1.0, len(qs), seed=args.seed + 7)
    lat, rows, cap_mk = srv.run_trace(cq, np.zeros(len(cq)))
    capacity = len(cq) / cap_mk
    serial_mk = float(service[cq].sum())          # the same requests, one at a time
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = R.kernel_launches()
    sampler.mark_start()
    per_rate = []
    for frac in (0.2, 0.4, 0.6, 0.8, 0.95):
        rate = frac * capacity
        tq, ta = W.served_trace(n_rate, rate, len(qs), seed=args.seed + int(frac * 100))
        st0 = srv.stats()
        lat, rows, mk = srv.run_trace(tq, ta)
        st1 = srv.stats()
        n_done = max(1, st1["completed"] - st0["completed"])
        scanned = float(q_rows[tq].sum())
        # serial plain execution of the same arrivals: one request at a time, in arrival order
        done = 0.0
        slat = np.zeros(len(tq))
        for k, (qq, a) in enumerate(zip(tq, ta)):
            done = max(done, a) + service[qq]
            slat[k] = done - a
        s_mk = done - ta[0]
        per_rate.append({
            "rate_rps": rate, "fraction_of_served_capacity": frac, "requests": int(len(tq)),
            "served": {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                       "rows_per_s": scanned / mk, "requests_per_s": len(tq) / mk,
                       "mean_queue_ms": (st1["queue_s"] - st0["queue_s"]) / n_done * 1e3,
                       "mean_run_ms": (st1["run_s"] - st0["run_s"]) / n_done * 1e3,
                       "solo_requests": st1["solo"] - st0["solo"]},
            "serial_plain": {"p50_ms": float(np.percentile(slat, 50) * 1e3),
                             "p99_ms": float(np.percentile(slat, 99) * 1e3),
                             "rows_per_s": scanned / s_mk, "requests_per_s": len(tq) / s_mk},
        })
    sampler.mark_end()
    clocks = sampler.stop()
    launches = R.kernel_launches() - launches0
    st = srv.stats()
    top = per_rate[-1]
    out = {
        "metric": METRIC, "value": top["served"]["rows_per_s"], "unit": "rows/s", "n_gpus": world,
        "steps": len(per_rate), "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32/int64/f32/f64/date32 (VM registers int64/f64)",
        "data": "synthetic (seeded, generated on the GPU)",
        "config": served_config(args, world),
        "capacity": {"requests": int(len(cq)), "arrivals": "all at once",
                     "served_rps": capacity, "serial_plain_rps": len(cq) / serial_mk,
                     "served_rows_per_s": float(q_rows[cq].sum() / cap_mk),
                     "serial_plain_rows_per_s": float(q_rows[cq].sum() / serial_mk),
                     "speedup_vs_serial_plain": serial_mk / cap_mk},
        "per_rate": per_rate,
        "server": dict(st, start_s=round(start_s, 2), generate_s=round(gen_s, 2)),
        "gpu_launches": int(launches), "clocks": clocks, "e2e": None,
        "e2e_note": "served tables are resident in HBM by design; requests carry no host data",
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    srv.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload in ("batched", "served"):
        threads = os.cpu_count() or 1
        fn = cpu_batched if args.workload == "batched" else cpu_served
        what = "programs of the mix" if args.workload == "batched" else "queries of the served workload"
        fn(threads, 8, 20_000, args.seed)
        times = [fn(threads, 64 if args.workload == "batched" else 32, 200_000, args.seed)
                 for _ in range(max(1, min(args.steps, 5)))]
        rows = times[0][0]
        t = statistics.mean(x[1] for x in times)
        v = rows / t
        out = {"metric": METRIC, "value": v, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "int32/int64/f32/f64", "data": "synthetic (seeded)",
               "impl": "reference",
               "config": batched_config(args, world) if args.workload == "batched" else served_config(args, world),
               "cpu_baseline": {"value": v, "unit": "rows/s", "cores": threads, "kind": "port",
                                "sample": f"first {64 if args.workload == 'batched' else 32} {what}, "
                                          f"tables capped at 200000 rows ({rows} rows)"},
               "e2e": {"value": v, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out), flush=True)
        return
    n = args.rows or DEFAULT_ROWS[args.workload]
    threads = os.cpu_count() or 1
    # bounded sample per step, sized from a probe so the whole run stays within a few minutes
    sel = args.pattern if args.workload == "gather" else args.selectivity
    probe = min(n, 100_000 if args.workload == "scan_filter" else 1_000_000)
    dt = cpu_time(args.workload, probe, threads, sel)
    rows = int(min(n, max(probe, (probe / max(dt, 1e-9)) * 4.0)))
    for _ in range(args.warmup):
        cpu_time(args.workload, min(rows, probe), threads, sel)
    times = [cpu_time(args.workload, rows, threads, sel) for _ in range(args.steps)]
    t = sum(times) / len(times)
    v = rows / t
    out = {"metric": METRIC, "value": v, "unit": "rows/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None,
           "dtype": {"fused_project": "f64+int64", "filter_project": "f64+int64", "plain_vm": "f64+int64",
                     "filter_gather": "int32/int64/f32/f64/date32/bool8 gather",
                  "gather": "int32/int64/f32/f64/date32/bool8 gather",
                  "scan_filter": "u8 text -> int32/f64/date64",
                  "parquet_filter": "Parquet pages -> int32/f64/date64",
                  "parquet_dict_filter": "Parquet pages -> int32/f64/date64"}[args.workload],
           "data": "synthetic (seeded)", "impl": "reference",
           "config": workload_config(args.workload, n, sel, world),
           "cpu_baseline": {"value": v, "unit": "rows/s", "cores": threads, "kind": "port",
                            "sample": f"{rows} of {n} rows per step", "cpu_model": cpu_model()},
           "e2e": {"value": v, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fused_project",
                    choices=["fused_project", "plain_vm", "filter_gather", "filter_project", "gather", "batched",
                             "served", "scan_filter", "parquet_filter", "parquet_dict_filter"])
    ap.add_argument("--tables", type=int, default=24)
    ap.add_argument("--queries", type=int, default=96)
    ap.add_argument("--requests", type=int, default=50_000)
    ap.add_argument("--budget-gb", type=float, default=120.0)
    ap.add_argument("--waves", type=int, default=2)
    ap.add_argument("--wave-rows", type=int, default=0, help="served: rows per wave (0: the library default)")
    ap.add_argument("--programs", type=int, default=256)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--max-rows", type=int, default=0, help="batched: cap every table (profiling captures)")
    ap.add_argument("--floor-from-ncu", default=None,
                    help="batched: write profiles/batch_mix_fp64.json from an ncu CSV of the capped plain calls "
                         "(no GPU needed) and exit")
    ap.add_argument("--capped-rows", type=int, default=1_000_000,
                    help="batched: also compare batch and plain calls over the first N rows of every table")
    ap.add_argument("--selectivity", type=float, default=0.5)
    ap.add_argument("--pattern", default="permutation", choices=["permutation", "random", "sorted"],
                    help="gather: the index column's pattern")
    ap.add_argument("--rows", type=int, default=0)
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-parity", action="store_true", help="skip the full-size oracle check")
    ap.add_argument("--no-extra", action="store_true",
                    help="default run: measure only the default workload, not the extra blocks")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.floor_from_ncu:
        table = floor_table_from_ncu(args.floor_from_ncu, args.programs, args.seed, args.max_rows or 200_000)
        with open(os.path.join(ROOT, "profiles", "batch_mix_fp64.json"), "w") as f:
            json.dump(table, f, indent=0)
        print(json.dumps(batch_floor(table, 2070.0, load_peaks()[0])))
        return
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "served":
        run_served(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
