#!/usr/bin/env python3
"""Benchmark of the GB300 row-wise filter+project evaluator.

Default workload: the deep plan (frozen 12-level CASE/COALESCE/MOD/FLOOR/LN/EXP
projection + 2-conjunct filter) over 2^28 rows x 6 nullable columns, one batch
per step, inputs resident in HBM (2^28 rows >> the 129 MB L2, so no L2 flush is
needed between steps).

JSON line (rank 0):
  value     rows/s, inputs resident on the device, whole job over all ranks
  e2e       rows/s through gx_plan_execute_host with pinned HOST buffers: H2D of
            the step's inputs + evaluation + D2H of the outputs inside the timed
            region (the library overlaps them by row chunk)
  roofline  algorithmic bytes of the fused filter+project kernel / its average
            CUDA-event duration vs the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (scalar restatement of the reference's
            interpreter, all host threads) on a bounded sample of the same workload

``--impl reference`` times the reference's CPU implementation of the path: the
reference's GPU interpreter needs libcudf 21.08, which is not installable
offline, so the oracle port (a C++ restatement of it) runs on the host cores.
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
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def profile_traffic(kernel_key: str):
    """Per-row DRAM traffic of the fused kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{kernel_key}.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_row:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []          # (host time, csv line)
        self.window = None       # (start, end) of the timed region

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def wait_first_sample(self, timeout=10.0):
        t0 = time.time()
        while self.proc and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.05)

    def mark(self, start, end):
        self.window = (start, end)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.window:
            inside = [x for x in lines if self.window[0] - 0.15 <= x[0] <= self.window[1] + 0.15]
            if inside:
                lines = inside
        for _, ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_sample_rate(name, w, sample_rows, nthreads, min_seconds=10.0, seed=7):
    """Oracle rows/s on a bounded host sample of the workload (repeat >= min_seconds)."""
    from blazingsql_gb300 import workloads as W
    from oracle import pyoracle
    cols = W.host_columns(name, sample_rows, seed=seed)
    pyoracle.filter_project(cols, w.condition, w.projections, nthreads, 0)  # warm (parse, page-in)
    t0 = time.perf_counter()
    reps = 0
    while True:
        pyoracle.filter_project(cols, w.condition, w.projections, nthreads, 0)
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or reps >= 1000:
            break
    return sample_rows * reps / el, reps, el


def full_parity(name, w, cols, stream):
    """The whole step's output against the oracle on the same rows: validity
    and integer data bit for bit, float data bit for bit except, for the deep
    plan, the rows whose CASE branch goes through LN / EXP (CUDA's log / exp
    against glibc, within 2 ulp)."""
    import numpy as np
    import blazingsql_gb300 as g
    from blazingsql_gb300 import workloads as W
    from blazingsql_gb300.types import is_float
    from oracle import pyoracle
    out = g.filter_project(cols, w.condition, w.projections, stream=stream)
    got = [c.to_host() for c in out]
    g.api.free_columns(out, stream)
    host = W.device_to_host(cols)
    t0 = time.perf_counter()
    exp, rows = pyoracle.filter_project(host, w.condition, w.projections, os.cpu_count() or 1, 0)
    oracle_s = time.perf_counter() - t0
    loose = W.c2_transcendental_rows(host) if name == "c2" else np.zeros(rows, dtype=bool)
    ok = len(got) == len(exp) and all(a.size == rows for a in got)
    bad_rows, worst = 0, 0.0
    for a, b in zip(got, exp):
        if not ok:
            break
        va, vb = a.valid(), b.valid()
        bad = va != vb
        x, y = a.values(), b.values()
        if is_float(a.type_id):
            it = np.int64 if x.dtype == np.float64 else np.int32
            xi, yi = x.view(it).astype(np.int64), y.view(it).astype(np.int64)
            xi = np.where(xi < 0, np.int64(-2**63) - xi, xi) if it == np.int64 else xi
            yi = np.where(yi < 0, np.int64(-2**63) - yi, yi) if it == np.int64 else yi
            d = np.abs(xi - yi).astype(np.float64)
            nan_ok = np.isnan(x) == np.isnan(y)
            d = np.where(np.isnan(x) & np.isnan(y), 0.0, d)
            bad |= vb & ((~loose & (d != 0)) | ~nan_ok | (loose & (d > 2)))
            if (vb & loose).any():
                worst = max(worst, float(d[vb & loose].max()))
        else:
            bad |= vb & (x != y)
        bad_rows += int(bad.sum())
    del host, got, exp
    return {"rows": w.rows, "out_rows": int(rows), "matches_oracle": bool(ok and bad_rows == 0),
            "mismatched_rows": bad_rows, "transcendental_rows": int(loose.sum()),
            "max_ulp_transcendental_rows": worst, "exact_elsewhere": True, "oracle_seconds": oracle_s}


def run_reference(args, world, rank):
    """CPU reference arm: the oracle port on all host cores, rank 0 only, on
    the same rows as our arm (the full workload unless --ref-rows is set)."""
    if rank != 0:
        return
    from blazingsql_gb300 import workloads as W
    w = W.workload(args.config, args.rows or None)
    nthreads = os.cpu_count() or 1
    sample = args.ref_rows or w.rows
    from oracle import pyoracle
    cols = W.host_columns(args.config, sample, seed=7)
    for _ in range(args.warmup):
        pyoracle.filter_project(cols, w.condition, w.projections, nthreads, 0)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        pyoracle.filter_project(cols, w.condition, w.projections, nthreads, 0)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = sample * args.steps / total
    line = {
        "impl": "reference", "metric": "filter_project_rows_per_s", "value": value, "unit": "rows/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic",
        "config": {"workload": w.name, "rows_per_step": sample, "rows_of_workload": w.rows,
                   "host_threads": nthreads},
        "cpu_baseline": {"value": value, "unit": "rows/s", "cores": nthreads, "kind": "port",
                         "sample": f"{sample} rows of {w.name} per step, the whole step's rows (the reference's GPU "
                                   f"interpreter needs libcudf 21.08, not installable offline; the oracle restates "
                                   f"it in C++)"},
        "e2e": {"value": value, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batched_compare(nbatches: int = 512, seed: int = 3, reps: int = 3):
    """C3: the deep plan over execution-graph batches of log-uniform size in
    [1K, 4M] rows, (a) one gx_plan_execute call per batch, as the batched
    execution graph calls the filter, and (b) the batch runner: one persistent
    kernel in a captured CUDA graph with an autotuned block shape.  Both read
    the same resident batches; outputs are library-allocated and freed."""
    import torch
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300 import workloads as W
    sizes = W.c3_batch_sizes(seed, nbatches)
    total = sum(sizes)
    w = W.workload("c2", total)
    stream = torch.cuda.current_stream()
    cols = W.device_columns("c2", total, seed=seed)
    batches = W.slice_batches(cols, sizes)
    plan = g.Plan(w.schema, w.condition, w.projections)
    torch.cuda.synchronize()

    def per_batch():
        rows = []
        for b in batches:
            out, r = plan.execute(b, stream=stream)
            rows.append(r)
            g.api.free_columns(out, stream)
        return rows

    per_batch()  # compile + warm
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    rows_a = per_batch()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_a = e0.elapsed_time(e1)
    # per-size-bucket rate of the per-batch path
    buckets = {"1K-16K": [0, 0.0], "16K-256K": [0, 0.0], "256K-4M": [0, 0.0]}
    import time
    for b, n in zip(batches, sizes):
        key = "1K-16K" if n < 16384 else ("16K-256K" if n < 262144 else "256K-4M")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out, _ = plan.execute(b, stream=stream)
        g.api.free_columns(out, stream)
        torch.cuda.synchronize()
        buckets[key][0] += n
        buckets[key][1] += time.perf_counter() - t0
    runner = g.BatchRunner(plan, nbatches, total, autotune=True)
    L = N.lib()
    nout = plan.num_outputs

    def runner_pass(bound, count):
        """One runner call over bound batches (library-allocated outputs, freed
        with one call); returns the rows per batch."""
        outs, rows = runner.run(bound, stream=stream, raw=True)
        g.api.free_column_array(outs, count * nout, stream)
        return rows

    def runner_time(bound, count):
        """(call ms, kernel ms) per run: the call through the C ABI with its
        output allocation, descriptor upload, graph launch, readback and free,
        and the persistent kernel alone (CUDA events around it)."""
        runner_pass(bound, count)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            runner_pass(bound, count)
        e1.record(stream)
        torch.cuda.synchronize()
        call_ms = e0.elapsed_time(e1) / reps
        L.gx_debug_kernel_ms(1)
        L.gx_debug_set_kernel_timing(1)
        try:
            for _ in range(reps):
                runner_pass(bound, count)
        finally:
            L.gx_debug_set_kernel_timing(0)
        return call_ms, L.gx_debug_kernel_ms(1) / reps

    bound_all = runner.bind(batches)
    rows_b = runner_pass(bound_all, nbatches)  # tunes on this first run
    ms_b, kms_b = runner_time(bound_all, nbatches)
    rows_b = runner_pass(bound_all, nbatches)
    bt, words = runner.config()
    # the batch stream: the persistent kernel fed batch by batch while it runs
    # (each push from this Python loop: ctypes argument building plus three
    # asynchronous copies), with the runner's tuned shape; timed from the
    # kernel's launch to the returned outputs
    bstream = g.BatchStream(plan, nbatches, total, block_threads=bt, words_per_warp=words)

    def stream_pass():
        bstream.start(stream)
        for b in batches:
            bstream.push(b)
        out = bstream.finish()
        g.api.free_columns([c for cols, _ in out for c in cols], stream)
        return [r for _, r in out]

    rows_s = stream_pass()
    stream_ms = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        stream_pass()
        stream_ms.append((time.perf_counter() - t0) * 1e3)
    ms_s = min(stream_ms)
    del bstream
    # the runner's own rate per batch-size bucket: the same runner over the
    # bucket's batches alone
    runner_buckets = {}
    for key, lo, hi in (("1K-16K", 0, 16384), ("16K-256K", 16384, 262144), ("256K-4M", 262144, 1 << 40)):
        sel = [b for b, n in zip(batches, sizes) if lo <= n < hi]
        nrows = sum(n for n in sizes if lo <= n < hi)
        if not sel:
            continue
        cms, kms = runner_time(runner.bind(sel), len(sel))
        runner_buckets[key] = {"batches": len(sel), "rows": nrows, "rows_per_s": nrows / (cms / 1e3),
                               "kernel_rows_per_s": nrows / (kms / 1e3)}
    del batches, cols
    torch.cuda.empty_cache()
    return {
        "runner_bucket_rows_per_s": runner_buckets,
        "workload": f"c3_batched_deep_plan: {nbatches} batches, log-uniform 1K-4M rows, {total} rows in all",
        "runner_rows_per_s": total / (ms_b / 1e3), "per_batch_calls_rows_per_s": total / (ms_a / 1e3),
        "runner_vs_per_batch_calls": ms_a / ms_b, "runner_ms": ms_b, "per_batch_calls_ms": ms_a,
        "runner_kernel_ms": kms_b, "runner_kernel_rows_per_s": total / (kms_b / 1e3),
        "stream_rows_per_s": total / (ms_s / 1e3), "stream_ms": ms_s, "stream_identical_row_counts": rows_s == rows_b,
        "identical_row_counts": rows_a == rows_b,
        "autotuned": {"block_threads": bt, "words_per_warp": words, "vector_width": 1},
        "per_batch_calls_bucket_rows_per_s": {k: (v[0] / v[1] if v[1] > 0 else None) for k, v in buckets.items()},
    }


def single_config(name: str, rows: int, reps: int = 10):
    """One configuration's fused filter + project over resident inputs, one
    batch per call: rows/s and the kernel's HBM fraction (CUDA events around
    the kernel inside the library)."""
    import torch
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300 import workloads as W
    L = N.lib()
    stream = torch.cuda.current_stream()
    w = W.workload(name, rows)
    cols = W.device_columns(name, rows, seed=1)
    torch.cuda.synchronize()

    def step():
        out = g.filter_project(cols, w.condition, w.projections, stream=stream)
        r = out[0].size
        g.api.free_columns(out, stream)
        return r

    for _ in range(6):  # warm-up: JIT and the plan's block-shape trials (a warm-up and four candidates)
        out_rows = step()
    torch.cuda.synchronize()
    L.gx_debug_kernel_ms(1)
    L.gx_debug_set_kernel_timing(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        out_rows = step()
    e1.record(stream)
    torch.cuda.synchronize()
    L.gx_debug_set_kernel_timing(0)
    kms = L.gx_debug_kernel_ms(1) / reps
    ms = e0.elapsed_time(e1) / reps
    alg = w.algorithmic_bytes(rows, out_rows)
    peak, _ = measured_peak_hbm()
    del cols
    torch.cuda.empty_cache()
    return {"workload": f"{w.name}: {rows} rows, one batch per call", "rows_per_s": rows / (ms / 1e3),
            "ms_per_call": ms, "kernel_ms": kms, "out_rows": out_rows,
            "roofline": {"bound": "hbm", "achieved": alg / (kms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / (kms / 1e3) / 1e9 / peak, "algorithmic_bytes": alg}}


def c5_batches(rows: int = 600_000_000, batch_rows: int = 1 << 22, reps: int = 3):
    """The order-line configuration as it is specified: 600M rows in 4M-row
    batches (the last one partial), run by the batch runner (one persistent
    kernel for all batches in a captured CUDA graph), beside one
    gx_plan_execute call per batch; inputs resident, outputs library-owned."""
    import torch
    import blazingsql_gb300 as g
    from blazingsql_gb300 import workloads as W
    stream = torch.cuda.current_stream()
    w = W.workload("c5", rows)
    cols = W.device_columns("c5", rows, seed=5)
    sizes = [batch_rows] * (rows // batch_rows) + ([rows % batch_rows] if rows % batch_rows else [])
    batches = W.slice_batches(cols, sizes)
    plan = g.Plan(w.schema, w.condition, w.projections)
    torch.cuda.synchronize()
    runner = g.BatchRunner(plan, len(sizes), rows, autotune=True)
    bound = runner.bind(batches)
    nout = plan.num_outputs
    outs, r = runner.run(bound, stream=stream, raw=True)  # tunes on this first run
    g.api.free_column_array(outs, len(sizes) * nout, stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        outs, r = runner.run(bound, stream=stream, raw=True)
        g.api.free_column_array(outs, len(sizes) * nout, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_runner = e0.elapsed_time(e1) / reps
    out_rows = sum(r)
    for b in batches[:6]:  # warm the per-call path: its block-shape tuning tries four candidates
        o, _ = plan.execute(b, stream=stream)
        g.api.free_columns(o, stream)
    torch.cuda.synchronize()
    e0.record(stream)
    calls_rows = 0
    for b in batches:
        o, rr = plan.execute(b, stream=stream)
        calls_rows += rr
        g.api.free_columns(o, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_calls = e0.elapsed_time(e1)
    alg = w.algorithmic_bytes(rows, out_rows)
    peak, _ = measured_peak_hbm()
    bt, words = runner.config()
    del batches, cols, runner
    torch.cuda.empty_cache()
    return {"workload": f"{w.name}: {rows} rows in {len(sizes)} batches of {batch_rows} rows",
            "runner_rows_per_s": rows / (ms_runner / 1e3), "runner_ms": ms_runner,
            "per_batch_calls_rows_per_s": rows / (ms_calls / 1e3), "per_batch_calls_ms": ms_calls,
            "identical_row_counts": calls_rows == out_rows, "out_rows": out_rows,
            "runner_hbm_frac": alg / (ms_runner / 1e3) / 1e9 / peak,
            "autotuned": {"block_threads": bt, "words_per_warp": words}}


def aggregate_compare(rows: int, seed: int = 5, reps: int = 5):
    """Fused filter + group-by aggregation (gx_filter_aggregate) on the
    order-line columns with TPC-H Q1's aggregation shape (C5 condition, keys
    $5, $6, nine aggregations), inputs resident: rows/s and HBM GB/s of the
    aggregation kernel against the measured peak.  Beside it the unfused
    chain: gx_filter_project materialises the keys and aggregation inputs, and
    gx_filter_aggregate reads them back; and the C5 filter + projection alone.
    A sample's groups are checked against the CPU oracle."""
    import numpy as np
    import torch
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300 import workloads as W
    from blazingsql_gb300.types import is_float, unpack_validity
    L = N.lib()
    stream = torch.cuda.current_stream()
    w = W.workload("c5", rows)
    cols = W.device_columns("c5", rows, seed=seed)
    torch.cuda.synchronize()

    def timed(fn):
        for _ in range(6):  # warm-up: JIT and the plan's block-shape trials (a warm-up and four candidates)
            fn()
        torch.cuda.synchronize()
        L.gx_debug_kernel_ms(1)
        L.gx_debug_set_kernel_timing(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        L.gx_debug_set_kernel_timing(0)
        return e0.elapsed_time(e1) / reps, L.gx_debug_kernel_ms(1) / reps

    def agg():
        out, groups = g.filter_aggregate(cols, W.C5_CONDITION, W.C5_AGG_KEYS, W.C5_AGGREGATIONS, stream=stream)
        g.api.free_columns(out, stream)

    # unfused: the filter + projection materialises the keys and the
    # aggregation inputs, then an aggregation reads them back
    nk = len(W.C5_AGG_KEYS)
    mat = [f"${c}" for c in W.C5_AGG_KEYS]
    agg2 = []
    for kind, e in W.C5_AGGREGATIONS:
        if e and e not in mat:
            mat.append(e)
        agg2.append((kind, f"${mat.index(e)}" if e else ""))

    def unfused():
        out = g.filter_project(cols, W.C5_CONDITION, mat, stream=stream)
        res, _ = g.filter_aggregate(out, None, list(range(nk)), agg2, stream=stream)
        g.api.free_columns(res, stream)
        g.api.free_columns(out, stream)

    def fp():
        out = g.filter_project(cols, W.C5_CONDITION, W.C5_PROJECTIONS, stream=stream)
        g.api.free_columns(out, stream)

    agg_ms, agg_kernel_ms = timed(agg)
    unfused_ms, unfused_kernel_ms = timed(unfused)
    fp_ms, fp_kernel_ms = timed(fp)
    in_bytes = rows * w.in_bytes_per_row
    peak, peak_kind = measured_peak_hbm()
    achieved = in_bytes / (agg_kernel_ms / 1e3) / 1e9
    # parity on a sample: the groups of the first 2^18 rows against the oracle
    from oracle import agg_ref
    from blazingsql_gb300.types import HostColumn, np_dtype
    ns = min(rows, 1 << 18)
    out, groups = g.filter_aggregate(W.slice_batches(cols, [ns])[0], W.C5_CONDITION, W.C5_AGG_KEYS,
                                     W.C5_AGGREGATIONS, stream=stream)
    got = [c.to_host() for c in out]
    g.api.free_columns(out, stream)
    sample = []
    for c in cols:  # the first ns rows only
        dt = np_dtype(c.type_id)
        data = c.data[:ns * dt.itemsize].cpu().numpy().view(dt).copy()
        mask = None if c.mask is None else c.mask[:((ns + 31) // 32) * 4].cpu().numpy().view(np.uint32).copy()
        sample.append(HostColumn(c.type_id, data, mask))
    exp = agg_ref.filter_aggregate(sample, W.C5_CONDITION, W.C5_AGG_KEYS, W.C5_AGGREGATIONS)
    ok = groups == len(exp[0].data)
    if ok:
        nk = len(W.C5_AGG_KEYS)
        keyset = lambda cs: [tuple(int(cs[j].data[r]) for j in range(nk)) for r in range(len(cs[0].data))]
        order = sorted(range(groups), key=lambda r: keyset(got)[r])
        for x, y in zip(got, exp):
            dx = np.asarray(x.data[:groups])[order]
            dy = np.asarray(y.data[:groups])
            vx = unpack_validity(x.mask, groups)[order]
            vy = unpack_validity(y.mask, groups)
            ok &= bool(np.array_equal(vx, vy))
            if is_float(x.type_id):
                ok &= bool(np.allclose(dx[vx], dy[vy], rtol=1e-9, atol=0))
            else:
                ok &= bool(np.array_equal(dx[vx], dy[vy]))
    del cols
    torch.cuda.empty_cache()
    return {
        "workload": f"c5_q1_filter_aggregate: {rows} rows, 7 columns, keys $5 $6, 9 aggregations",
        "rows_per_s": rows / (agg_ms / 1e3), "ms": agg_ms, "kernel_ms": agg_kernel_ms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "algorithmic_bytes": in_bytes},
        "groups": groups, "oracle_sample_rows": ns, "matches_oracle": bool(ok),
        "filter_project_rows_per_s": rows / (fp_ms / 1e3), "filter_project_ms": fp_ms,
        "filter_project_kernel_ms": fp_kernel_ms,
        "unfused_ms": unfused_ms, "unfused_kernel_ms": unfused_kernel_ms,
        "fused_vs_unfused": unfused_ms / agg_ms,
    }


def _string_column(torch, gen, phrases, rows, device):
    """A cudf-layout string column whose rows are drawn from `phrases` (built on the device)."""
    from blazingsql_gb300.api import DeviceColumn
    from blazingsql_gb300.types import TypeId
    width = max(len(p) for p in phrases)
    tab = torch.zeros((len(phrases), width), dtype=torch.uint8)
    for i, ph in enumerate(phrases):
        tab[i, :len(ph)] = torch.tensor(list(ph.encode()), dtype=torch.uint8)
    tab = tab.to(device)
    plen = torch.tensor([len(ph) for ph in phrases], dtype=torch.int32, device=device)
    ids = torch.randint(0, len(phrases), (rows,), generator=gen, device=device)
    lens = plen[ids]
    offs = torch.zeros(rows + 1, dtype=torch.int32, device=device)
    offs[1:] = torch.cumsum(lens, 0, dtype=torch.int32)
    keep = torch.arange(width, device=device, dtype=torch.int32)[None, :] < lens[:, None]
    chars = torch.masked_select(tab[ids], keep)
    del keep
    return DeviceColumn(TypeId.STRING, chars if chars.numel() else torch.zeros(1, dtype=torch.uint8, device=device),
                        None, 0, rows, offs)


STRING_CONDITION = "AND(<=($4, 1998-09-02), NOT(LIKE($8, '%ke%q%')))"
STRING_PROJECTIONS = ["$7", "SUBSTRING($8, 1, 10)", "CONCAT($7, '-', CAST($0):VARCHAR)",
                      "*(*($1, -(100, $2)), +(100, $3))"]


def strings_compare(rows: int, seed: int = 6, reps: int = 5):
    """String columns on the path: the order-line columns plus a mode column
    (7 short tokens) and a comment column (10-43 characters of random words),
    filtered by a date and a LIKE on the comment, projecting the mode
    (gathered), SUBSTRING of the comment, CONCAT of the mode with a formatted
    integer, and the exact charge.  Inputs resident; the whole
    gx_filter_project call is timed (string pre-pass, plan kernel, string
    builders), its compulsory bytes against the measured HBM peak.  A sample
    is checked against the CPU oracle and timed there."""
    import numpy as np
    import torch
    import blazingsql_gb300 as g
    from blazingsql_gb300 import workloads as W
    from blazingsql_gb300.types import HostColumn, TypeId, np_dtype
    rng = np.random.default_rng(seed)
    letters = np.array(list("abcdefghijklmnopqrstuvwxyz"))
    words = ["".join(rng.choice(letters, int(rng.integers(3, 10)))) for _ in range(200)]
    comments = []
    while len(comments) < 512:
        ph = ""
        target = int(rng.integers(10, 44))
        while len(ph) < target:
            ph = (ph + " " + words[int(rng.integers(0, len(words)))]).strip()
        comments.append(ph[:target].strip() or "x")
    modes = ["".join(rng.choice(letters, int(rng.integers(3, 8)))).upper() for _ in range(7)]
    stream = torch.cuda.current_stream()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    cols = W.device_columns("c5", rows, seed=seed) + [_string_column(torch, gen, modes, rows, "cuda"),
                                                      _string_column(torch, gen, comments, rows, "cuda")]
    torch.cuda.synchronize()

    def fp():
        return g.filter_project(cols, STRING_CONDITION, STRING_PROJECTIONS, stream=stream)

    for _ in range(6):  # warm-up: JIT and the plan's block-shape trials (a warm-up and four candidates)
        g.api.free_columns(fp(), stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        out = fp()
        g.api.free_columns(out, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    out = fp()
    kept = out[0].size
    # compulsory bytes: the referenced columns once, every output once
    used = [0, 1, 2, 3, 4, 7, 8]
    in_bytes = 0
    for i in used:
        c = cols[i]
        in_bytes += c.data.numel() + (c.str_offsets.numel() * 4 if c.str_offsets is not None else 0)
    out_bytes = 0
    for c in out:
        out_bytes += (c._c.string_bytes + 4 * (c.size + 1)) if c.type_id == TypeId.STRING else \
            c.size * np_dtype(c.type_id).itemsize
        out_bytes += (c.size + 7) // 8
    g.api.free_columns(out, stream)
    peak, peak_kind = measured_peak_hbm()
    achieved = (in_bytes + out_bytes) / (ms / 1e3) / 1e9
    # the first ns rows against the oracle, and the oracle's rate on them
    import time
    from oracle import strings_ref
    ns = min(rows, 1 << 14)
    sample = W.slice_batches(cols, [ns])[0]
    got = g.filter_project(sample, STRING_CONDITION, STRING_PROJECTIONS, stream=stream)
    hc, hs = [], {}
    for i, c in enumerate(cols):
        if c.type_id == TypeId.STRING:
            o = c.str_offsets[:ns + 1].cpu().numpy()
            ch = c.data[:int(o[-1])].cpu().numpy().tobytes()
            hs[i] = [ch[o[r]:o[r + 1]].decode() for r in range(ns)]
            hc.append(None)
        else:
            dt = np_dtype(c.type_id)
            hc.append(HostColumn(c.type_id, c.data[:ns * dt.itemsize].cpu().numpy().view(dt).copy()))
    t0 = time.time()
    exp, erows = strings_ref.filter_project(hc, hs, STRING_CONDITION, STRING_PROJECTIONS, nthreads=1)
    oracle_s = time.time() - t0
    ok = got[0].size == erows
    for gc, ec in zip(got, exp):
        if not ok:
            break
        if gc.type_id == TypeId.STRING:
            ok = gc.to_strings() == ec
        else:
            h = gc.to_host()
            ok = bool(np.array_equal(np.asarray(h.data[:erows]), np.asarray(ec.data[:erows])))
    g.api.free_columns(got, stream)
    del cols
    torch.cuda.empty_cache()
    return {
        "workload": f"order-line columns + 2 string columns: {rows} rows; filter {STRING_CONDITION}; "
                    f"projections {STRING_PROJECTIONS}",
        "rows_per_s": rows / (ms / 1e3), "ms": ms, "selectivity": kept / rows,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "algorithmic_bytes": in_bytes + out_bytes},
        "oracle_sample_rows": ns, "matches_oracle": bool(ok), "oracle_rows_per_s": ns / oracle_s,
    }


def learned_compare(batches: int, rows: int, seed: int = 4):
    """C4: the skewed 6-conjunct filter over `batches` batches of `rows` rows,
    through gx_learner under four policies on the same resident batches:
    plain fixed-order two-pass, textual-order single pass (no network), learned
    (order from device memory, full-size outputs) and learned_sized (outputs of
    the predicted size, allocated as each batch's prediction is read); the
    learned ones include the labelled warm-up and relabel batches (the plain
    fixed-order evaluator in one pass that counts each conjunct's passes) and
    the training.  Rows/s per
    policy over the whole batch stream, timed around one
    gx_learner_execute_batches call (the C ABI call a C++ caller makes; the
    Python argument building and result wrapping stay outside) and, for
    reference, through one gx_learner_execute per batch from Python.  Per-batch
    row counts and sampled full outputs must agree exactly across policies."""
    import numpy as np
    import torch
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300 import workloads as W
    w = W.workload("c4")
    stream = torch.cuda.current_stream()
    data = [W.c4_batch_device(rows, seed, b) for b in range(batches)]
    torch.cuda.synchronize()
    plan = g.Plan(w.schema, w.condition, w.projections, nullable=[False] * 8)
    # learned: order from device memory, full-size outputs (no host round trip);
    # learned_sized: prediction read back, outputs of the predicted size
    policies = {"plain": (N.GX_LEARN_POLICY_PLAIN, 1), "textual": (N.GX_LEARN_POLICY_TEXTUAL, 1),
                "learned": (N.GX_LEARN_POLICY_LEARNED, 0), "learned_sized": (N.GX_LEARN_POLICY_LEARNED, 1)}
    # compile every kernel variant and grow the allocation pool once, outside
    # the timed passes
    for pol, sized in policies.values():
        lr = g.Learner(plan, policy=pol, warmup_batches=1, relabel_every=0, fast_words_per_warp=8,
                       size_outputs=sized)
        for cols, _, _ in lr.execute_batches(data, stream=stream):
            g.api.free_columns(cols, stream)
    torch.cuda.synchronize()
    res = {}
    counts = {}
    check_batches = (0, batches // 2, batches - 1)
    sampled = {}
    L = N.lib()
    for name, (pol, sized) in policies.items():
        def learner():
            # trained online on its first 4 batches (labelled by the plain
            # fixed-order pass), then the network alone orders the rest
            return g.Learner(plan, policy=pol, async_training=1, warmup_batches=4, relabel_every=0,
                             fast_words_per_warp=8, size_outputs=sized)
        # the batch queue in one native call (what the execution graph's C++
        # kernel does), each next batch prepared while the current one runs
        lr = learner()
        q = lr.queue_args(data)
        l0 = L.gx_debug_launch_count()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        lr.run_queue(q, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        launches = L.gx_debug_launch_count() - l0
        out = lr.queue_results(q)
        infos = [i for _, _, i in out]
        counts[name] = [r for _, r, _ in out]
        for b, (cols, _, _) in enumerate(out):
            if b in check_batches:
                sampled.setdefault(b, []).append([c.to_host() for c in cols])
            g.api.free_columns(cols, stream)
        del out, lr
        # the same queue driven from Python, one gx_learner_execute per batch
        lr = learner()
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        if pol == N.GX_LEARN_POLICY_LEARNED:
            lr.prepare(data[0], stream=stream)
        for b in range(batches):
            if pol == N.GX_LEARN_POLICY_LEARNED and b + 1 < batches:
                lr.prepare(data[b + 1], stream=stream)  # look-ahead: next batch's prediction
            cols, r, _ = lr.execute(data[b], stream=stream)
            if r != counts[name][b]:
                counts[name][b] = -1
            g.api.free_columns(cols, stream)
        p1.record(stream)
        torch.cuda.synchronize()
        py_ms = p0.elapsed_time(p1)
        del lr
        res[name] = {"rows_per_s": rows * batches / (ms / 1e3), "ms": ms, "launches": launches,
                     "python_loop_rows_per_s": rows * batches / (py_ms / 1e3), "python_loop_ms": py_ms}
        if name.startswith("learned"):
            res[name].update({
                "plain_batches": sum(1 for i in infos if i["path"] == 0),
                "reruns": sum(i["reruns"] for i in infos),
                "final_train_loss": infos[-1]["train_loss"],
                "orders_used": len({tuple(i["order"]) for i in infos if i["path"] == 1}),
            })
    identical = counts["plain"] == counts["textual"] == counts["learned"] == counts["learned_sized"]
    # full outputs of the sampled batches, every policy against the plain one
    for b, per_policy in sampled.items():
        for other in per_policy[1:]:
            for x, y in zip(per_policy[0], other):
                identical &= bool(np.array_equal(x.data.view(np.uint8), y.data.view(np.uint8)))
                identical &= bool(np.array_equal(x.mask, y.mask))
    checks = len(sampled)
    del data
    torch.cuda.empty_cache()
    return {
        "workload": f"c4_learned_order_filter: {batches} batches x {rows} rows, 8 Zipf(1.2) columns, 6 AND conjuncts",
        "plain_rows_per_s": res["plain"]["rows_per_s"], "textual_rows_per_s": res["textual"]["rows_per_s"],
        "learned_rows_per_s": res["learned"]["rows_per_s"],
        "learned_sized_rows_per_s": res["learned_sized"]["rows_per_s"],
        "learned_vs_plain": res["learned"]["rows_per_s"] / res["plain"]["rows_per_s"],
        "learned_sized_vs_plain": res["learned_sized"]["rows_per_s"] / res["plain"]["rows_per_s"],
        "learned_vs_textual": res["learned"]["rows_per_s"] / res["textual"]["rows_per_s"],
        "identical_output": identical, "row_counts_checked": batches, "full_outputs_checked": checks,
        "detail": res,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c5"])
    ap.add_argument("--rows", type=int, default=0, help="override rows per step")
    ap.add_argument("--cpu-sample-rows", type=int, default=1 << 22)
    ap.add_argument("--ref-rows", type=int, default=0, help="reference arm rows per step (default: the workload's)")
    ap.add_argument("--parity", type=int, default=1, help="compare the whole step's output with the oracle")
    ap.add_argument("--c1-rows", type=int, default=1 << 24, help="C1 rows (0 skips the C1 key)")
    ap.add_argument("--c5-rows", type=int, default=600_000_000, help="C5 rows (0 skips the C5 key)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--mode", type=int, default=-1, help="filter mode override (0 auto, 1 two-pass, 2 single)")
    ap.add_argument("--learned-batches", type=int, default=64, help="C4 batches (0 skips the learned comparison)")
    ap.add_argument("--learned-rows", type=int, default=1 << 22, help="C4 rows per batch")
    ap.add_argument("--batched-batches", type=int, default=512, help="C3 batches (0 skips the batched comparison)")
    ap.add_argument("--string-rows", type=int, default=1 << 25,
                    help="rows of the string-column filter + project (0 skips it)")
    ap.add_argument("--agg-rows", type=int, default=1 << 27,
                    help="rows of the fused filter + aggregation measurement (0 skips it)")
    args = ap.parse_args()
    # at least 3 warm-up steps, and enough for the block-shape tuner of the
    # library's single-pass filter to have measured its four candidates (its
    # first large call is a warm-up, the next four try one candidate each)
    args.warmup = max(3 if args.impl == "reference" else 6, args.warmup)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch
    if args.mode >= 0:
        os.environ["GX_FILTER_MODE"] = str(args.mode)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300 import workloads as W

    w = W.workload(args.config, args.rows or None)
    n = w.rows
    stream = torch.cuda.current_stream()
    cols = W.device_columns(args.config, n, seed=1 + rank)
    torch.cuda.synchronize()
    L = N.lib()

    def step():
        out = g.filter_project(cols, w.condition, w.projections, stream=stream)
        rows = out[0].size
        g.api.free_columns(out, stream)
        return rows

    for _ in range(args.warmup):
        out_rows = step()
    torch.cuda.synchronize()

    # ---- device-resident timed region -------------------------------------
    L.gx_debug_kernel_ms(1)
    L.gx_debug_set_kernel_timing(1)
    launches0 = L.gx_debug_launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local).start()
    clocks.wait_first_sample()
    t_start = time.time()
    ev0.record(stream)
    for _ in range(args.steps):
        out_rows = step()
    ev1.record(stream)
    torch.cuda.synchronize()
    t_end = time.time()
    if t_end - t_start < 0.3:  # keep one more sampling period inside the window
        time.sleep(0.3)
    clocks.mark(t_start, t_end)
    clocks.stop()
    L.gx_debug_set_kernel_timing(0)
    kernel_ms_total = L.gx_debug_kernel_ms(1)
    launches = L.gx_debug_launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    rows_total = n * args.steps * world
    value = rows_total / (ms / 1e3)

    # roofline of the dominant kernel (fused filter+project)
    alg_bytes = w.algorithmic_bytes(n, out_rows)
    kernel_ms = kernel_ms_total / args.steps
    achieved_gbs = alg_bytes / (kernel_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic_per_row = profile_traffic(f"{args.config}_fused_filter_project")

    # ---- end to end: pinned host buffers, H2D + evaluate + D2H ------------
    # through gx_plan_execute_host: host columns in, host columns out; the
    # library pipelines the copies in, the kernels and the copies out by chunk
    e2e = None
    if rank == 0 or world > 1:
        from blazingsql_gb300.types import np_dtype
        host_in = []
        h2d = 0
        for c in cols:
            hd = torch.empty(c.data.numel(), dtype=torch.uint8, pin_memory=True)
            hd.copy_(c.data)
            hm = None
            if c.mask is not None:
                hm = torch.empty(c.mask.numel(), dtype=torch.uint8, pin_memory=True)
                hm.copy_(c.mask)
            host_in.append((c.type_id, hd, hm))
            h2d += n * np_dtype(c.type_id).itemsize + (((n + 31) // 32) * 4 if hm is not None else 0)
        hplan = g.Plan(w.schema, w.condition, w.projections)
        otypes = hplan.output_types()
        host_out = [(torch.empty(n * np_dtype(t).itemsize + 64, dtype=torch.uint8, pin_memory=True),
                     torch.empty(((n + 31) // 32) * 4 + 64, dtype=torch.uint8, pin_memory=True)) for t in otypes]
        views = [(t, hd.data_ptr(), hm.data_ptr() if hm is not None else 0, n) for t, hd, hm in host_in]
        outs = [(hb.data_ptr(), hmk.data_ptr(), n) for hb, hmk in host_out]

        def e2e_step():
            rows = hplan.execute_host(views, outs, stream=stream)
            return sum(rows * np_dtype(t).itemsize + (rows + 31) // 32 * 4 for t in otypes)

        e2e_step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.e2e_steps):
            d2h = e2e_step()
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1) / args.e2e_steps
        e2e = {"value": n / (e2e_ms / 1e3) * world, "unit": "rows/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms, "api": "gx_plan_execute_host"}
        del host_in, host_out, hplan

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # ---- parity of the whole step against the oracle -------------------------
    parity = full_parity(args.config, w, cols, stream) if args.parity else None

    batched = None
    if args.batched_batches > 0:
        if cols is not None:
            del cols
            cols = None
            torch.cuda.empty_cache()
        batched = batched_compare(args.batched_batches)
    aggregate = None
    if args.agg_rows > 0:
        if cols is not None:
            del cols
            cols = None
            torch.cuda.empty_cache()
        aggregate = aggregate_compare(args.agg_rows)
    strings = None
    if args.string_rows > 0:
        if cols is not None:
            del cols
            cols = None
            torch.cuda.empty_cache()
        strings = strings_compare(args.string_rows)
    c1 = None
    if args.c1_rows > 0:
        if cols is not None:
            del cols
            cols = None
            torch.cuda.empty_cache()
        c1 = single_config("c1", args.c1_rows)
    c5 = None
    if args.c5_rows > 0:
        if cols is not None:
            del cols
            cols = None
            torch.cuda.empty_cache()
        c5 = {"single_call": single_config("c5", min(args.c5_rows, 1 << 28)), "batched": c5_batches(args.c5_rows)}
    learned = None
    if args.learned_batches > 0:
        if cols is not None:
            del cols
            cols = None
            torch.cuda.empty_cache()
        learned = learned_compare(args.learned_batches, args.learned_rows)

    # ---- CPU baseline: oracle on a bounded sample --------------------------
    nthreads = os.cpu_count() or 1
    cpu_rate, reps, el = cpu_sample_rate(args.config, w, min(args.cpu_sample_rows, n), nthreads,
                                         args.cpu_seconds)
    line = {
        "metric": "filter_project_rows_per_s", "value": value, "unit": "rows/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic",
        "config": {"workload": w.name, "rows_per_step": n, "out_rows_per_step": out_rows,
                   "selectivity": out_rows / n, "columns": len(w.schema),
                   "l2": "inputs (>10 GB/step) far larger than the 129 MB L2; no flush needed",
                   "filter_mode": os.environ.get("GX_FILTER_MODE", "auto")},
        "hbm_gbs": alg_bytes * args.steps / (ms / 1e3) / 1e9,
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peak, "unit": "GB/s",
                     "frac": achieved_gbs / peak, "peak_source": peak_kind,
                     "traffic": None if traffic_per_row is None else traffic_per_row * n,
                     "algorithmic_bytes": alg_bytes, "kernel_ms": kernel_ms},
        "cpu_baseline": {"value": cpu_rate, "unit": "rows/s", "cores": nthreads, "kind": "port",
                         "sample": f"{min(args.cpu_sample_rows, n)} rows of {w.name}, {reps} reps in {el:.1f} s"},
        "e2e": e2e,
        "parity": parity,
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "batched": batched,
        "learned": learned,
        "aggregate": aggregate,
        "strings": strings,
        "c1": c1,
        "c5": c5,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
