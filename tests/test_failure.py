"""Bounded device waits give up and report GX_ERR_TIMEOUT instead of hanging.

The failure is made on the host: the filter's tile ticket starts past tile 0,
so tile 0 is never claimed and never publishes its look-back status, and every
later tile's look-back can only run out of polls.  No GPU fault, trap or endless
loop is involved; after the timed-out call the device must still evaluate a
plan correctly."""
import os

import numpy as np
import pytest

import blazingsql_gb300 as g
from blazingsql_gb300 import _native as N
from blazingsql_gb300 import workloads as W
from tests.helpers import OracleEngine, assert_tables_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tma", ["0", "1"])
def test_lookback_wait_gives_up(monkeypatch, tma):
    monkeypatch.setenv("GX_TMA", tma)  # direct-load kernel and tile-staged kernel
    w = W.workload("c1", 20_000)
    cols = [g.api.DeviceColumn.from_host(c) for c in W.host_columns("c1", 20_000, seed=3)]
    plan = g.Plan(w.schema, w.condition, w.projections)
    # tiles of at most 1024 rows: 20,000 rows are many tiles, tile 0 never claimed
    rc = plan.wait_test(cols, first_tile=1, spin_limit=2000)
    assert rc == N.GX_ERR_TIMEOUT
    # the device and the library still work: the same plan, normally, against the oracle
    out, rows = plan.execute(cols)
    got = [c.to_host() for c in out]
    exp = OracleEngine(4).filter_project(W.host_columns("c1", 20_000, seed=3), w.condition, w.projections)
    assert rows == exp[0].size
    assert_tables_equal(got, exp, what="after a timed-out call")


def test_no_timeout_without_skipped_tiles():
    w = W.workload("c1", 20_000)
    cols = [g.api.DeviceColumn.from_host(c) for c in W.host_columns("c1", 20_000, seed=4)]
    plan = g.Plan(w.schema, w.condition, w.projections)
    assert plan.wait_test(cols, first_tile=0, spin_limit=0) == N.GX_OK
