"""gx_plan_execute_noalloc: the filter + project entry point that allocates no
device memory (for callers whose own pool owns the device budget, or whose
per-batch path must not enter an allocator).  Its results must equal those of
the regular entry point, gx_plan_execute, call after call: the fixed scratch
array it shares across calls keeps the previous call's contents, so two
different batches in a row also check that it is cleared.

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import blazingsql_gb300 as g
from blazingsql_gb300 import _native as N
from blazingsql_gb300 import workloads as W
from blazingsql_gb300.types import HostColumn, np_dtype
from tests.helpers import assert_tables_equal

pytestmark = pytest.mark.gpu


def _caller_buffers(torch, types, capacity):
    """Output buffers owned by the test (the entry point must not allocate)."""
    keep, cols = [], []
    mask_bytes = max(64, (capacity + 511) // 512 * 64)
    for t in types:
        d = torch.zeros(max(64, capacity * np_dtype(t).itemsize), dtype=torch.uint8, device="cuda")
        m = torch.zeros(mask_bytes, dtype=torch.uint8, device="cuda")
        keep += [d, m]
        cols.append(N.Column(t, 0, d.data_ptr(), m.data_ptr(), 0, capacity))
    return keep, cols


def _to_host(col: N.Column) -> HostColumn:
    dt = np_dtype(col.type_id)
    data = np.empty(max(1, col.size), dtype=dt)
    mask = np.zeros(max(16, ((col.size + 31) // 32 + 15) // 16 * 16), dtype=np.uint32)
    st = N.StatusInfo()
    N.check(N.lib().gx_column_to_host(C.byref(col), data.ctypes.data, mask.ctypes.data, None, C.byref(st)), st)
    return HostColumn(col.type_id, data[:col.size], mask)


@pytest.mark.parametrize("workload", ["c1", "c2"])
def test_noalloc_matches_regular_entry_point(workload):
    torch = pytest.importorskip("torch")
    w = W.workload(workload)
    plan = g.Plan(w.schema, w.condition, w.projections)
    for n, seed in ((100_003, 1), (40_000, 2)):  # two calls in a row, different batches
        cols = W.host_columns(workload, n, seed=seed)
        dev = [g.DeviceColumn.from_host(c) for c in cols]
        ref, ref_rows = plan.execute(dev)
        expected = [c.to_host() for c in ref]
        keep, bufs = _caller_buffers(torch, plan.output_types(), n)
        # any device allocation made by the library now would fail
        from blazingsql_gb300.api import fail_next_allocation
        fail_next_allocation(1)
        try:
            got, rows = plan.execute_noalloc(dev, bufs)
        finally:
            fail_next_allocation(0)
        assert rows == ref_rows
        # the same kernel runs on both paths: results are bit-identical
        assert_tables_equal([_to_host(c) for c in got], expected, what=f"{workload} n={n}")
        del keep


def _tile_rows():
    """Rows per tile of the no-allocation path: its configured block shape."""
    import os
    return int(os.environ.get("GX_WARPS") or 4) * int(os.environ.get("GX_WORDS") or 4) * 32


def test_noalloc_capacity_too_small_writes_nothing_past_the_buffers():
    torch = pytest.importorskip("torch")
    w = W.workload("c1")
    plan = g.Plan(w.schema, w.condition, w.projections)
    n = 50_000
    cols = W.host_columns("c1", n, seed=9)
    dev = [g.DeviceColumn.from_host(c) for c in cols]
    _, need = plan.execute(dev)
    cap = need // 2
    canary, keep, bufs = 64, [], []
    for t in plan.output_types():
        dbytes = cap * np_dtype(t).itemsize
        mbytes = max(64, (cap + 511) // 512 * 64)
        d = torch.full((dbytes + canary,), 0xAB, dtype=torch.uint8, device="cuda")
        m = torch.full((mbytes + canary,), 0xAB, dtype=torch.uint8, device="cuda")
        keep.append((d, m, dbytes, mbytes))
        bufs.append(N.Column(t, 0, d.data_ptr(), m.data_ptr(), 0, cap))
    keep_v: list = []
    views, nc = g.api._views(dev, keep_v)
    outs = (N.Column * len(bufs))(*bufs)
    rows = C.c_int64(0)
    st = N.StatusInfo()
    rc = N.lib().gx_plan_execute_noalloc(plan._h, views, nc, outs, C.byref(rows), None, C.byref(st))
    assert rc == N.GX_ERR_CAPACITY
    assert rows.value == need
    for d, m, dbytes, mbytes in keep:
        assert (d[dbytes:].cpu().numpy() == 0xAB).all(), "data written past the caller's buffer"
        assert (m[mbytes:].cpu().numpy() == 0xAB).all(), "mask written past the caller's buffer"


def test_noalloc_rejects_oversized_batch():
    torch = pytest.importorskip("torch")
    w = W.workload("c1")
    plan = g.Plan(w.schema, w.condition, w.projections)
    tiny = torch.zeros(64, dtype=torch.uint8, device="cuda")
    too_many = N.GX_NOALLOC_MAX_TILES * _tile_rows() + 1
    views = [g.DeviceColumn(t, tiny, None, 0, too_many) for t in w.schema]
    keep, bufs = _caller_buffers(torch, plan.output_types(), 16)
    with pytest.raises(g.GxError) as ei:
        plan.execute_noalloc(views, bufs)  # rejected on the host before any device work
    assert ei.value.code == N.GX_ERR_INVALID
    assert "no-allocation scratch" in ei.value.message
    del keep
