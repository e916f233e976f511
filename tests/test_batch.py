"""Batch runner: a table of batches through one persistent kernel in a captured
CUDA graph must return, for every batch, exactly what the single-batch plan
returns for it (and what the CPU oracle returns)."""
from __future__ import annotations

import numpy as np
import pytest

from blazingsql_gb300 import workloads as W
from blazingsql_gb300.types import TypeId as T

from helpers import OracleEngine, assert_tables_equal


def _host(cols):
    return [c.to_host() for c in cols]


def test_c3_batch_sizes_are_log_uniform():
    sizes = W.c3_batch_sizes()
    assert len(sizes) == 512
    assert min(sizes) >= 1024 and max(sizes) < 4194304
    total = sum(sizes)
    assert 200_000_000 < total < 330_000_000
    # log-uniform: about a third of the batches below 16K rows
    assert 120 < sum(1 for n in sizes if n < 16384) < 220


def test_batched_kernel_compiles():
    import blazingsql_gb300 as g
    w = W.workload("c2", 1024)
    plan = g.Plan(w.schema, w.condition, w.projections)
    src = plan.kernel_source(6, [True] * 6)
    assert "tile_base" in src and "GxBatchHdr" in src
    plan.compile_check(6, [True] * 6)
    plan.compile_check(6, [False] * 6)


@pytest.mark.gpu
@pytest.mark.parametrize("workload", ["c1", "c2", "c5"])
def test_runner_matches_single_batch_plan(workload):
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    rng = np.random.default_rng(5)
    sizes = [0, 1, 31, 32, 33, 511, 512, 513, 1000, 4097] + [int(x) for x in np.exp(rng.uniform(0, np.log(30000), 20))]
    total = sum(sizes)
    w = W.workload(workload, total)
    host = W.host_columns(workload, total, seed=11)
    dev = [DeviceColumn.from_host(c) for c in host]
    batches = W.slice_batches(dev, sizes)
    plan = g.Plan(w.schema, w.condition, w.projections)
    runner = g.BatchRunner(plan, max_batches=64, max_total_rows=total, autotune=False)
    got, rows = runner.run(batches)
    oracle = OracleEngine(nthreads=4)
    start = 0
    for b, n in enumerate(sizes):
        exp, erows = plan.execute(batches[b])
        assert rows[b] == erows, (b, n)
        assert_tables_equal(_host(got[b]), _host(exp), what=f"{workload} batch {b} ({n} rows)")
        if b in (0, 1, 9, len(sizes) - 1):
            sl = [g.HostColumn(c.type_id, c.data[start:start + n],
                               None if c.mask is None else g.pack_validity(
                                   g.unpack_validity(c.mask, start + n)[start:]))
                  for c in host]
            ref = oracle.filter_project(sl, w.condition, w.projections)
            assert_tables_equal(_host(got[b]), ref, ulps=2, what=f"oracle {workload} batch {b}")
        start += n
    # a second run (graph replay) over a different set of batches
    got2, rows2 = runner.run(batches[5:15])
    for i, b in enumerate(range(5, 15)):
        assert rows2[i] == rows[b]
        assert_tables_equal(_host(got2[i]), _host(got[b]))


@pytest.mark.gpu
def test_runner_caller_buffers_and_autotune():
    import torch
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    n_total = (1 << 20) + 12345
    sizes = [n_total // 4, n_total // 4, n_total - 2 * (n_total // 4)]
    w = W.workload("c1", n_total)
    dev = W.device_columns("c1", n_total, seed=4)
    batches = W.slice_batches(dev, sizes)
    plan = g.Plan(w.schema, w.condition, w.projections)
    runner = g.BatchRunner(plan, max_batches=8, max_total_rows=n_total, autotune=True)
    got, rows = runner.run(batches)
    bt, words = runner.config()
    assert (bt // 32, words) in [(4, 2), (4, 4), (4, 8), (8, 2), (8, 4), (2, 8), (1, 16)]
    keep = []
    bufs = []
    for b, n in enumerate(sizes):
        for t in plan.output_types():
            width = np.dtype(g.types.np_dtype(t)).itemsize
            d = torch.full((max(n, 1) * width,), 0xAB, dtype=torch.uint8, device="cuda")
            m = torch.full((((n + 511) // 512) * 64 + 64,), 0xFF, dtype=torch.uint8, device="cuda")
            keep += [d, m]
            c = N.Column()
            c.type_id, c.data, c.null_mask, c.size, c.capacity = t, d.data_ptr(), m.data_ptr(), 0, n
            bufs.append(c)
    got2, rows2 = runner.run(batches, out=bufs)
    assert rows2 == rows
    for b in range(len(sizes)):
        exp, erows = plan.execute(batches[b])
        assert erows == rows[b]
        assert_tables_equal(_host(got[b]), _host(exp))
        for j, c in enumerate(got2[b]):
            nc = g.NativeColumn(c)
            try:
                assert_tables_equal([nc.to_host()], [_host(exp)[j]], what=f"caller buffers batch {b} output {j}")
            finally:
                nc._c.data = None  # caller-owned memory: not freed by the library
    del keep


@pytest.mark.gpu
def test_runner_limits():
    import blazingsql_gb300 as g
    w = W.workload("c1", 5000)
    dev = W.device_columns("c1", 5000, seed=2)
    plan = g.Plan(w.schema, w.condition, w.projections)
    runner = g.BatchRunner(plan, max_batches=2, max_total_rows=4000, autotune=False)
    with pytest.raises(g.GxError):
        runner.run(W.slice_batches(dev, [1000, 1000, 1000]))  # too many batches
    with pytest.raises(g.GxError):
        runner.run(W.slice_batches(dev, [3000, 2000]))  # too many rows
    got, rows = runner.run(W.slice_batches(dev, [3000, 1000]))
    assert len(got) == 2
    nofilter = g.Plan([T.INT64], None, ["$0"])
    with pytest.raises(g.GxError):
        g.BatchRunner(nofilter, 4, 100)
