"""Host-to-host execution (gx_plan_execute_host): the chunked copy/compute
pipeline returns exactly what the device entry point returns for the same
plan (bit-exact data and validity), across chunk boundaries, with nulls, for
the fallback plans (literal outputs, no condition, two-pass mode) and for the
capacity and empty-input edge cases; one case is also checked against the
CPU oracle."""
import numpy as np
import pytest

import blazingsql_gb300 as g
from blazingsql_gb300 import _native as N
from blazingsql_gb300 import workloads as W
from blazingsql_gb300.types import HostColumn, TypeId as T, np_dtype

from helpers import OracleEngine, assert_tables_equal

pytestmark = pytest.mark.gpu


def _run_host(plan, cols, capacity=None):
    n = cols[0].data.shape[0] if cols else 0
    cap = n if capacity is None else capacity
    outs = [(np.zeros(max(cap, 1), dtype=np_dtype(t)), np.zeros(max(1, (cap + 31) // 32), dtype=np.uint32))
            for t in plan.output_types()]
    views = [(c.type_id, c.data.ctypes.data, c.mask.ctypes.data if c.mask is not None else 0, n) for c in cols]
    rows = plan.execute_host(views, [(d.ctypes.data, m.ctypes.data, cap) for d, m in outs])
    return [HostColumn(t, d[:rows], m) for t, (d, m) in zip(plan.output_types(), outs)], rows


def _run_device(plan, cols):
    from blazingsql_gb300.api import DeviceColumn
    dev = [DeviceColumn.from_host(c) for c in cols]
    got, rows = plan.execute(dev)
    return [c.to_host() for c in got], rows


def _same(a, b, rows, what):
    assert len(a) == len(b)
    nw = (rows + 31) // 32
    for j, (x, y) in enumerate(zip(a, b)):
        assert np.array_equal(x.data[:rows].view(np.uint8), y.data[:rows].view(np.uint8)), f"{what}: data of output {j}"
        xm = x.mask[:nw].copy()
        ym = y.mask[:nw].copy()
        if rows % 32:
            keep = np.uint32((1 << (rows % 32)) - 1)
            xm[-1] &= keep
            ym[-1] &= keep
        assert np.array_equal(xm, ym), f"{what}: validity of output {j}"


@pytest.mark.parametrize("name,n", [("c2", 3 * (1 << 22) + 12345), ("c1", 5 * (1 << 22) + 1), ("c5", 70_001),
                                    ("c2", 31)])
def test_host_pipeline_matches_device(name, n):
    """Several chunks (the row ranges of chunk k+1 start where chunk k's end,
    mid-word in the output masks) against the device entry point."""
    w = W.workload(name)
    cols = W.host_columns(name, n, seed=17)
    plan = g.Plan(w.schema, w.condition, w.projections)
    got, rows = _run_host(plan, cols)
    exp, erows = _run_device(plan, cols)
    assert rows == erows
    _same(got, exp, rows, f"{name} n={n}")


def test_host_pipeline_matches_oracle():
    cols = W.host_columns("c1", 100_003, seed=5)
    plan = g.Plan(W.workload("c1").schema, W.C1_CONDITION, W.C1_PROJECTIONS)
    got, rows = _run_host(plan, cols)
    exp = OracleEngine(nthreads=8).filter_project(cols, W.C1_CONDITION, W.C1_PROJECTIONS)
    assert rows == len(exp[0].data)
    assert_tables_equal(got, exp, what="host pipeline vs oracle")


@pytest.mark.parametrize("cond,exprs,mode", [
    ("<($0, 50)", ["$0", "7", "+($1, 1.5)"], N.GX_FILTER_AUTO),      # literal output: whole-table form
    (None, ["*($0, 3)", "$1"], N.GX_FILTER_AUTO),                     # no condition
    ("<($0, 50)", ["$0", "+($1, 1.5)"], N.GX_FILTER_TWO_PASS),        # two-pass mode
])
def test_host_fallback_forms(cond, exprs, mode):
    rng = np.random.default_rng(3)
    n = 9000
    x0 = rng.integers(0, 100, n).astype(np.int64)
    x1 = rng.normal(0, 10, n)
    valid = rng.random(n) > 0.1
    cols = [HostColumn(T.INT64, x0, g.pack_validity(valid)), HostColumn(T.FLOAT64, x1)]
    plan = g.Plan([T.INT64, T.FLOAT64], cond, exprs, filter_mode=mode)
    got, rows = _run_host(plan, cols)
    exp, erows = _run_device(plan, cols)
    assert rows == erows
    _same(got, exp, rows, f"{cond} {exprs}")


def test_host_capacity_and_empty():
    w = W.workload("c1")
    cols = W.host_columns("c1", 1 << 20, seed=2)
    plan = g.Plan(w.schema, w.condition, w.projections)
    _, rows = _run_host(plan, cols)
    with pytest.raises(N.GxError, match=f"needed rows={rows}"):
        _run_host(plan, cols, capacity=rows - 1)
    got, rows2 = _run_host(plan, cols, capacity=rows)
    assert rows2 == rows
    empty = [HostColumn(c.type_id, c.data[:0], None if c.mask is None else c.mask[:1]) for c in cols]
    got, r0 = _run_host(plan, empty)
    assert r0 == 0 and all(len(c.data) == 0 for c in got)
