"""Batch stream: one persistent kernel fed batch by batch while it runs.  Every
batch's output must equal what the single-batch plan returns for it; batches
pushed with host pauses in between (the kernel waiting on an empty queue) must
come out the same; a session that pushes nothing ends cleanly; a kernel kept
waiting past its limit reports GX_ERR_TIMEOUT and the object then works again."""
from __future__ import annotations

import time

import numpy as np
import pytest

from blazingsql_gb300 import workloads as W

from helpers import assert_tables_equal


def _host(cols):
    return [c.to_host() for c in cols]


def test_stream_kernel_compiles():
    import blazingsql_gb300 as g
    w = W.workload("c2", 1024)
    plan = g.Plan(w.schema, w.condition, w.projections)
    src = plan.kernel_source(9, [True] * 6)
    assert "claim_" in src and "wait_polls" in src and "GX_BATCH(pb)" in src
    plan.compile_check(9, [True] * 6)


def _batches(workload, sizes, seed):
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    total = sum(sizes)
    w = W.workload(workload, total)
    dev = [DeviceColumn.from_host(c) for c in W.host_columns(workload, total, seed=seed)]
    return g.Plan(w.schema, w.condition, w.projections), W.slice_batches(dev, sizes)


@pytest.mark.gpu
@pytest.mark.parametrize("workload", ["c1", "c2", "c5"])
def test_stream_matches_single_batch_plan(workload):
    import blazingsql_gb300 as g
    rng = np.random.default_rng(7)
    sizes = [0, 1, 31, 32, 33, 511, 512, 513, 1000, 4097] + [int(x) for x in np.exp(rng.uniform(0, np.log(60000), 20))]
    plan, batches = _batches(workload, sizes, 13)
    stream = g.BatchStream(plan, max_batches=64, max_total_rows=sum(sizes))
    stream.start()
    for b, batch in enumerate(batches):
        assert stream.push(batch) == b
        if b % 7 == 3:
            time.sleep(0.002)  # the kernel waits on an empty queue meanwhile
    out = stream.finish()
    assert len(out) == len(sizes)
    for b, (cols, rows) in enumerate(out):
        exp, erows = plan.execute(batches[b])
        assert rows == erows, (b, sizes[b])
        assert_tables_equal(_host(cols), _host(exp), what=f"{workload} batch {b} ({sizes[b]} rows)")
    # a second session on the same object, other batches, another block shape object
    stream.start()
    for batch in batches[10:20]:
        stream.push(batch)
    out2 = stream.finish()
    for i, (cols, rows) in enumerate(out2):
        assert rows == out[10 + i][1]
        assert_tables_equal(_host(cols), _host(out[10 + i][0]))


@pytest.mark.gpu
def test_stream_empty_session_and_limits():
    import blazingsql_gb300 as g
    plan, batches = _batches("c1", [5000, 7000], 3)
    stream = g.BatchStream(plan, max_batches=2, max_total_rows=12000, block_threads=64, words_per_warp=8)
    stream.start()
    assert stream.finish() == []
    stream.start()
    stream.push(batches[0])
    stream.push(batches[1])
    with pytest.raises(g.GxError):
        stream.push(batches[0])  # a third batch: more than the stream was created for
    out = stream.finish()
    assert [r for _, r in out] == [plan.execute(b)[1] for b in batches]
    with pytest.raises(g.GxError):
        stream.finish()  # not running


@pytest.mark.gpu
def test_stream_wait_limit_gives_up_then_recovers():
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    plan, batches = _batches("c1", [3000, 4000], 4)
    stream = g.BatchStream(plan, max_batches=4, max_total_rows=7000)
    stream.set_wait_polls(200)  # about 0.4 ms
    stream.start()
    time.sleep(0.2)  # nothing comes: every block gives up
    stream.push(batches[0])
    with pytest.raises(g.GxError) as ei:
        stream.finish()
    assert ei.value.code == N.GX_ERR_TIMEOUT
    stream.set_wait_polls(1 << 22)
    stream.start()
    for b in batches:
        stream.push(b)
    out = stream.finish()
    for b, (cols, rows) in enumerate(out):
        exp, erows = plan.execute(batches[b])
        assert rows == erows
        assert_tables_equal(_host(cols), _host(exp))
