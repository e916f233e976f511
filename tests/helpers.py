"""Shared test helpers: engines (oracle / GPU), column comparison, data makers."""
from __future__ import annotations

import math
from typing import List, Optional, Sequence

import numpy as np

from blazingsql_gb300.types import HostColumn, TypeId, is_float, np_dtype


# ------------------------------------------------------------------ engines
class OracleEngine:
    name = "oracle"

    def __init__(self, nthreads: int = 2):
        from oracle import pyoracle
        self.o = pyoracle
        self.nthreads = nthreads

    def evaluate_expressions(self, cols, exprs, seed=0):
        return self.o.evaluate_expressions(cols, exprs, self.nthreads, seed)

    def process_filter(self, cols, query_part):
        return self.o.process_filter(cols, query_part, self.nthreads)

    def process_project(self, cols, query_part):
        return self.o.process_project(cols, query_part, self.nthreads)

    def filter_project(self, cols, cond, exprs, seed=0):
        return self.o.filter_project(cols, cond, exprs, self.nthreads, seed)[0]


class GpuEngine:
    name = "gpu"

    def __init__(self):
        import blazingsql_gb300 as g
        self.g = g

    def evaluate_expressions(self, cols, exprs, seed=0):
        return [c.to_host() for c in self.g.evaluate_expressions(cols, exprs)]

    def process_filter(self, cols, query_part):
        return [c.to_host() for c in self.g.process_filter(cols, query_part)]

    def process_project(self, cols, query_part):
        return [c.to_host() for c in self.g.process_project(cols, query_part)[0]]

    def filter_project(self, cols, cond, exprs, seed=0):
        return [c.to_host() for c in self.g.filter_project(cols, cond, exprs)]


# --------------------------------------------------------------- comparison
def ulp_distance(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Distance in units in the last place between float arrays (same dtype)."""
    if a.dtype == np.float32:
        ia, ib = a.view(np.int32).astype(np.int64), b.view(np.int32).astype(np.int64)
        ia = np.where(ia < 0, np.int64(-2**31) - ia, ia)
        ib = np.where(ib < 0, np.int64(-2**31) - ib, ib)
    else:
        ia, ib = a.view(np.int64), b.view(np.int64)
        ia = np.where(ia < 0, np.int64(-2**63) - ia, ia)
        ib = np.where(ib < 0, np.int64(-2**63) - ib, ib)
    d = np.abs(ia.astype(object) - ib.astype(object)) if a.size < 64 else np.abs(ia - ib)
    return np.asarray(d, dtype=np.float64)


def assert_columns_equal(got: HostColumn, exp: HostColumn, ulps: float = 0, what: str = "") -> None:
    """Bit-exact comparison of validity (rows < n) and of data on valid rows.

    For float columns ``ulps`` > 0 allows that many units in the last place
    (NaN must match NaN, infinities must match exactly)."""
    assert got.type_id == exp.type_id, f"{what}: type {got.type_id} != {exp.type_id}"
    assert got.size == exp.size, f"{what}: size {got.size} != {exp.size}"
    gv, ev = got.valid(), exp.valid()
    bad = np.nonzero(gv != ev)[0]
    assert bad.size == 0, f"{what}: validity differs at rows {bad[:10].tolist()}"
    g, e = got.values()[ev], exp.values()[ev]
    if is_float(got.type_id):
        gn, en = np.isnan(g), np.isnan(e)
        bad = np.nonzero(gn != en)[0]
        assert bad.size == 0, f"{what}: NaN mismatch at valid rows {bad[:10].tolist()}"
        g, e = g[~gn], e[~en]
        if ulps == 0:
            it = np.int64 if g.dtype == np.float64 else np.int32
            bad = np.nonzero(g.view(it) != e.view(it))[0]
            assert bad.size == 0, (f"{what}: {bad.size} float values differ, e.g. rows {bad[:5].tolist()}: "
                                   f"{g[bad[:5]].tolist()} vs {e[bad[:5]].tolist()}")
        else:
            d = ulp_distance(g, e)
            worst = float(d.max()) if d.size else 0.0
            assert worst <= ulps, f"{what}: max ulp distance {worst} > {ulps}"
    else:
        bad = np.nonzero(g != e)[0]
        assert bad.size == 0, (f"{what}: {bad.size} values differ, e.g. {g[bad[:5]].tolist()} vs "
                               f"{e[bad[:5]].tolist()}")


def assert_columns_mixed(got: HostColumn, exp: HostColumn, loose_rows: np.ndarray, ulps: float,
                         what: str = "") -> float:
    """Validity bit-exact everywhere; float data bit-exact on the valid rows
    outside ``loose_rows`` and within ``ulps`` on the valid rows inside it (the
    rows whose value comes from a transcendental).  Returns the largest ulp
    distance seen on the loose rows."""
    assert got.type_id == exp.type_id and got.size == exp.size, f"{what}: type/size differ"
    gv, ev = got.valid(), exp.valid()
    bad = np.nonzero(gv != ev)[0]
    assert bad.size == 0, f"{what}: validity differs at rows {bad[:10].tolist()}"
    loose = np.asarray(loose_rows, dtype=bool)
    exact = ev & ~loose
    it = np.int64 if got.values().dtype == np.float64 else np.int32
    g, e = got.values(), exp.values()
    bad = np.nonzero(exact & (g.view(it) != e.view(it)))[0]
    assert bad.size == 0, (f"{what}: {bad.size} exact rows differ, e.g. rows {bad[:5].tolist()}: "
                           f"{g[bad[:5]].tolist()} vs {e[bad[:5]].tolist()}")
    lv = ev & loose
    gl, el = g[lv], e[lv]
    gn, en = np.isnan(gl), np.isnan(el)
    assert np.array_equal(gn, en), f"{what}: NaN mismatch on transcendental rows"
    d = ulp_distance(gl[~gn], el[~en])
    worst = float(d.max()) if d.size else 0.0
    assert worst <= ulps, f"{what}: max ulp distance {worst} > {ulps} on transcendental rows"
    return worst


def assert_tables_equal(got: Sequence[HostColumn], exp: Sequence[HostColumn], ulps: float = 0,
                        what: str = "") -> None:
    assert len(got) == len(exp), f"{what}: {len(got)} columns vs {len(exp)}"
    for i, (g, e) in enumerate(zip(got, exp)):
        assert_columns_equal(g, e, ulps, f"{what} col {i}")


# --------------------------------------------------------------- data makers
NUMERIC_TYPES = [TypeId.INT8, TypeId.INT16, TypeId.INT32, TypeId.INT64, TypeId.UINT8, TypeId.UINT16,
                 TypeId.UINT32, TypeId.UINT64, TypeId.FLOAT32, TypeId.FLOAT64, TypeId.BOOL8]
SIGNED_NUMERIC_TYPES = [TypeId.INT8, TypeId.INT16, TypeId.INT32, TypeId.INT64, TypeId.FLOAT32, TypeId.FLOAT64,
                        TypeId.BOOL8]
TIMESTAMP_TYPES = [TypeId.TIMESTAMP_DAYS, TypeId.TIMESTAMP_SECONDS, TypeId.TIMESTAMP_MILLISECONDS,
                   TypeId.TIMESTAMP_MICROSECONDS, TypeId.TIMESTAMP_NANOSECONDS]
LITERAL_TYPE_TOKEN = {TypeId.INT8: "TINYINT", TypeId.INT16: "SMALLINT", TypeId.INT32: "INTEGER",
                      TypeId.INT64: "BIGINT", TypeId.FLOAT32: "FLOAT", TypeId.FLOAT64: "DOUBLE"}


def cast_values(t: int, values) -> np.ndarray:
    """static_cast<T>(v) for each integer / float value (C++ semantics)."""
    dt = np_dtype(t)
    if t == TypeId.BOOL8:
        return np.array([1 if v else 0 for v in values], dtype=np.uint8)
    if np.issubdtype(dt, np.integer):
        bits = dt.itemsize * 8
        out = []
        for v in values:
            v = int(v) % (1 << bits)
            if np.issubdtype(dt, np.signedinteger) and v >= (1 << (bits - 1)):
                v -= 1 << bits
            out.append(v)
        return np.array(out, dtype=dt)
    return np.array(values, dtype=np.float64).astype(dt)


def column(t: int, values, valid=None) -> HostColumn:
    return HostColumn(t, cast_values(t, values), None if valid is None else
                      __import__("blazingsql_gb300.types", fromlist=["pack_validity"]).pack_validity(
                          np.asarray(valid, dtype=bool)))


def random_table(rng: np.random.Generator, n: int, spec, null_frac: float = 0.0) -> List[HostColumn]:
    """spec: list of (type_id, low, high) -> uniform columns (floats N(0, high))."""
    from blazingsql_gb300.types import pack_validity
    cols = []
    for t, lo, hi in spec:
        dt = np_dtype(t)
        if is_float(t):
            v = rng.normal(lo, hi, n).astype(dt)
        elif t == TypeId.BOOL8:
            v = (rng.random(n) < 0.5).astype(np.uint8)
        else:
            v = rng.integers(lo, hi, n, dtype=np.int64).astype(dt)
        mask = None
        if null_frac > 0:
            mask = pack_validity(rng.random(n) >= null_frac)
        cols.append(HostColumn(t, v, mask))
    return cols
