"""Fused filter + group-by aggregation (gx_filter_aggregate) against the CPU
oracle (oracle/agg_ref.py, a restatement of GroupBy.cpp's aggregation step).

Keys, counts, integer sums, MIN / MAX and validity must match exactly;
floating-point sums and means, whose addition order on the GPU depends on
scheduling (as in cudf's hash aggregation), within a relative 1e-9.  Groups
come out of the GPU unordered and are sorted by key (NULL first) before the
comparison, as the oracle orders them."""
from __future__ import annotations

import numpy as np
import pytest

from blazingsql_gb300 import workloads as W
from blazingsql_gb300.types import HostColumn, TypeId as T, is_float, pack_validity, unpack_validity
from oracle import agg_ref

from helpers import random_table

SUM, SUM0, MIN, MAX, COUNT_VALID, COUNT_ALL, MEAN = range(7)

# the TPC-H Q1 shape over the order-line columns: group by the two flags
Q1_AGGS = W.C5_AGGREGATIONS


def _sorted(cols, nk):
    """Rows ordered by key tuple, NULL before any value."""
    n = len(cols[0].data) if cols else 0
    keys = []
    for r in range(n):
        kt = []
        for j in range(nk):
            ok = bool(unpack_validity(cols[j].mask, n)[r])
            kt.append((1, int(cols[j].data[r])) if ok else (0, 0))
        keys.append(tuple(kt))
    order = sorted(range(n), key=lambda r: keys[r])
    out = []
    for c in cols:
        v = unpack_validity(c.mask, n)[order]
        out.append(HostColumn(c.type_id, np.asarray(c.data[:n])[order], pack_validity(v)))
    return out


def _compare(got, exp, nk, what):
    assert len(got) == len(exp), what
    g = _sorted(got, nk)
    n = len(exp[0].data)
    assert len(g[0].data) == n, f"{what}: {len(g[0].data)} groups vs {n}"
    for i, (x, y) in enumerate(zip(g, exp)):
        assert x.type_id == y.type_id, f"{what} col {i}: type {x.type_id} vs {y.type_id}"
        vx, vy = unpack_validity(x.mask, n), unpack_validity(y.mask, n)
        assert np.array_equal(vx, vy), f"{what} col {i}: validity"
        dx, dy = np.asarray(x.data[:n])[vx], np.asarray(y.data[:n])[vy]
        if is_float(x.type_id):
            np.testing.assert_allclose(dx, dy, rtol=1e-9, atol=0, err_msg=f"{what} col {i}")
        else:
            assert np.array_equal(dx, dy), f"{what} col {i}: values"


# ------------------------------------------------------------------ CPU
def test_oracle_groupby_rules():
    """The oracle's rules on a hand-checked table: NULL keys group together,
    SUM / MIN / MAX / MEAN of a group without valid input are NULL, SUM0 is 0,
    COUNT(x) counts valid inputs and COUNT(*) rows; no keys -> one row."""
    k = HostColumn(T.INT32, np.array([1, 1, 2, 7, 2, 9], dtype=np.int32),
                   pack_validity(np.array([1, 1, 1, 0, 1, 0], dtype=bool)))
    v = HostColumn(T.INT64, np.array([10, 20, 5, 1, -3, 4], dtype=np.int64),
                   pack_validity(np.array([1, 1, 0, 1, 0, 1], dtype=bool)))
    aggs = [(SUM, "$1"), (SUM0, "$1"), (MIN, "$1"), (MAX, "$1"), (COUNT_VALID, "$1"), (COUNT_ALL, ""), (MEAN, "$1")]
    out = agg_ref.filter_aggregate([k, v], None, [0], aggs)
    n = len(out[0].data)
    assert n == 3
    val = [unpack_validity(c.mask, n) for c in out]
    assert list(val[0]) == [False, True, True]                  # NULL key group first
    assert list(out[0].data[1:]) == [1, 2]
    assert list(out[1].data) == [5, 30, 0] and list(val[1]) == [True, True, False]   # SUM
    assert list(out[2].data) == [5, 30, 0] and list(val[2]) == [True, True, True]    # SUM0
    assert list(out[3].data[:2]) == [1, 10] and list(out[4].data[:2]) == [4, 20]     # MIN / MAX
    assert list(out[5].data) == [2, 2, 0] and list(out[6].data) == [2, 2, 2]        # COUNT(x), COUNT(*)
    assert out[7].data[0] == 2.5 and out[7].data[1] == 15.0 and not val[7][2]      # MEAN
    one = agg_ref.filter_aggregate([k, v], "<($0, 0)", [], aggs)
    assert len(one[0].data) == 1
    assert list(unpack_validity(one[0].mask, 1)) == [False]     # SUM of nothing: NULL
    assert one[1].data[0] == 0 and one[5].data[0] == 0         # SUM0 and COUNT(*)


@pytest.mark.parametrize("keys,has_mask", [([5, 6], False), ([], True), ([0, 4, 5], True), ([6], False)])
def test_aggregate_kernel_compiles(keys, has_mask):
    """NVRTC builds the aggregation kernel for sm_103a (no GPU): registers and
    shared memory stay within one block's budget."""
    import blazingsql_gb300 as g
    w = W.workload("c5")
    regs, spill, smem = g.api.aggregate_check(w.schema, [has_mask] * 7, W.C5_CONDITION, keys, Q1_AGGS)
    assert 0 < regs <= 255 and smem <= 48 * 1024


# ------------------------------------------------------------------ GPU
def _run(cols, cond, keys, aggs):
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    dev = [DeviceColumn.from_host(c) for c in cols]
    out, groups = g.filter_aggregate(dev, cond, keys, aggs)
    host = [c.to_host() for c in out]
    assert all(len(c.data) == groups for c in host)
    return host


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 4097, 200_003, (1 << 22) + 5])
def test_q1_shaped_matches_oracle(n):
    cols = W.host_columns("c5", n, seed=8)
    got = _run(cols, W.C5_CONDITION, [5, 6], Q1_AGGS)
    exp = agg_ref.filter_aggregate(cols, W.C5_CONDITION, [5, 6], Q1_AGGS)
    _compare(got, exp, 2, f"q1 n={n}")


@pytest.mark.gpu
@pytest.mark.parametrize("null_frac", [0.0, 0.2])
def test_every_kind_with_nulls(null_frac):
    rng = np.random.default_rng(17)
    n = 150_001
    cols = random_table(rng, n, [(T.INT16, -3, 4), (T.INT64, -1000, 1000), (T.FLOAT64, 0.0, 50.0),
                                 (T.INT32, -50, 50), (T.BOOL8, 0, 2), (T.FLOAT32, 0.0, 3.0)], null_frac=null_frac)
    aggs = [(SUM, "$1"), (SUM0, "*($1, $3)"), (MIN, "$2"), (MAX, "$2"), (MIN, "$3"), (MAX, "$5"),
            (COUNT_VALID, "$2"), (COUNT_ALL, ""), (MEAN, "$1"), (MEAN, "+($2, 1.5)"), (SUM, "$2")]
    for keys in ([0], [0, 4], []):
        got = _run(cols, ">($3, -40)", keys, aggs)
        exp = agg_ref.filter_aggregate(cols, ">($3, -40)", keys, aggs)
        _compare(got, exp, len(keys), f"keys={keys} nulls={null_frac}")


@pytest.mark.gpu
def test_many_groups_spill_to_global_table():
    """More groups than a block's table holds, and more than the global
    table's first size (it grows and the pass repeats)."""
    rng = np.random.default_rng(5)
    n = 600_000
    k = HostColumn(T.INT64, rng.integers(0, 250_000, n).astype(np.int64) * 7919)
    v = HostColumn(T.INT32, rng.integers(-9, 9, n).astype(np.int32))
    aggs = [(SUM, "$1"), (COUNT_ALL, ""), (MAX, "$1")]
    got = _run([k, v], None, [0], aggs)
    exp = agg_ref.filter_aggregate([k, v], None, [0], aggs)
    _compare(got, exp, 1, "many groups")


@pytest.mark.gpu
def test_empty_and_errors():
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    cols = W.host_columns("c5", 1000, seed=3)
    aggs = [(SUM, "$1"), (COUNT_ALL, ""), (SUM0, "$2")]
    # nothing passes: no groups with keys, one row without
    got = _run(cols, "<($0, -5)", [5], aggs)
    assert len(got[0].data) == 0
    got = _run(cols, "<($0, -5)", [], aggs)
    exp = agg_ref.filter_aggregate(cols, "<($0, -5)", [], aggs)
    _compare(got, exp, 0, "empty, no keys")
    empty = [HostColumn(c.type_id, c.data[:0]) for c in cols]
    assert len(_run(empty, None, [5], aggs)[0].data) == 0
    # a floating-point key, and COUNT(*) given an input, are refused
    fcol = random_table(np.random.default_rng(1), 10, [(T.FLOAT64, 0.0, 1.0)])
    with pytest.raises(N.GxError, match="group columns"):
        g.filter_aggregate([g.api.DeviceColumn.from_host(c) for c in fcol], None, [0], [(COUNT_ALL, "")])
    with pytest.raises(N.GxError, match="COUNT"):
        _run(cols, None, [5], [(COUNT_ALL, "$1")])
