"""BlazingSQL's own known-answer vectors, checked on the oracle (CPU) and on the
GPU evaluator.

Vectors come from the reference's gtest sources (see tests/golden/
reference_vectors.json, produced by extract_reference_vectors.py, each entry
citing file:lines).  Where a reference test hand-encodes an interpreter plan
(interops_tests.cpp) the same plan is written as the RexNode expression it
encodes.  In the numeric tables here, string columns of the reference fixtures
are replaced by an unused INT32 column; the reference's string-table tests run
in test_strings.py.
"""
import json
import os

import numpy as np
import pytest

from blazingsql_gb300.types import HostColumn, TypeId as T, np_dtype, pack_validity
from tests.helpers import (LITERAL_TYPE_TOKEN, NUMERIC_TYPES, SIGNED_NUMERIC_TYPES, TIMESTAMP_TYPES, GpuEngine,
                           OracleEngine, assert_columns_equal, cast_values, column)

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.json")))


@pytest.fixture(params=["oracle", pytest.param("gpu", marks=pytest.mark.gpu)], scope="module")
def engine(request):
    return OracleEngine() if request.param == "oracle" else GpuEngine()


def expect(t, values, valid=None):
    return column(t, values, valid)


# --------------------------------------------------- interops_tests.cpp:199-278
@pytest.mark.parametrize("t", SIGNED_NUMERIC_TYPES)
def test_interops_numeric(engine, t):
    g = GOLD["interops_numeric"]
    r = np.arange(10)
    cols = [column(t, r * 2), column(t, r * 10), column(t, r * 20)]
    lit = "true" if t == T.BOOL8 else f"2:{LITERAL_TYPE_TOKEN[t]}"
    out = engine.evaluate_expressions(cols, ["+(*(+($0, $1), $2), $1)", f"+($1, {lit})"])
    assert_columns_equal(out[0], expect(t, g["expected_col1"]), what="col1")
    assert_columns_equal(out[1], expect(t, g["expected_col2"]), what="col2")


def ts_inputs(t, start_ms, stop_ms, rows):
    """The reference's timestamp iterator: time_point_cast from ms, then
    start + (range / rows) * i in the type's representation."""
    per_ms = {T.TIMESTAMP_DAYS: (86400000, None), T.TIMESTAMP_SECONDS: (1000, None),
              T.TIMESTAMP_MILLISECONDS: (1, None), T.TIMESTAMP_MICROSECONDS: (None, 1000),
              T.TIMESTAMP_NANOSECONDS: (None, 1000000)}[t]

    def cast(ms):
        div, mul = per_ms
        if div:
            q = abs(ms) // div
            return q if ms >= 0 else -q   # duration_cast truncates toward zero
        return ms * mul
    start, stop = cast(start_ms), cast(stop_ms)
    step = (stop - start) // rows
    return [start + step * i for i in range(rows)]


# --------------------------------------------------- interops_tests.cpp:294-455
@pytest.mark.parametrize("t", TIMESTAMP_TYPES)
def test_day_of_week(engine, t):
    g = GOLD["interops_day_of_week"]
    vals = ts_inputs(t, g["start_ms"], g["stop_ms"], g["rows"])
    cols = [column(t, vals)]
    exp = g["expected_days"] if t == T.TIMESTAMP_DAYS else g["expected_other"]
    out = engine.evaluate_expressions(cols, ["BL_DOW($0)"])
    assert_columns_equal(out[0], expect(T.INT16, exp))
    out = engine.process_project(cols, "LogicalProject(EXPR$0=[EXTRACT(FLAG(DOW), $0)])")
    assert_columns_equal(out[0], expect(T.INT16, exp))


# --------------------------------------------------- interops_tests.cpp:457-557
@pytest.mark.parametrize("t", TIMESTAMP_TYPES)
def test_timestamp_components(engine, t):
    g = GOLD["interops_timestamp_components"]
    vals = ts_inputs(t, g["start_ms"], g["stop_ms"], g["rows"])
    exp = g["days"] if t == T.TIMESTAMP_DAYS else g["other"]
    ops = ["BL_YEAR", "BL_MONTH", "BL_DAY", "BL_HOUR", "BL_MINUTE", "BL_SECOND", "BL_DOW"]
    out = engine.evaluate_expressions([column(t, vals)], [f"{op}($0)" for op in ops])
    for k, op in enumerate(ops):
        assert_columns_equal(out[k], expect(T.INT16, exp[f"col{k + 1}"]), what=op)


# --------------------------------------------------- process_project.cpp:16-199
def project_table(t):
    g = GOLD["project_inputs"]
    return [column(t, g["col1"], [1] * 7), column(T.INT32, [0] * 7), column(t, g["col3"], [1] * 7)]


@pytest.mark.parametrize("t", NUMERIC_TYPES)
def test_project_numeric(engine, t):
    g = GOLD["project_inputs"]
    tab = project_table(t)
    out = engine.process_project(tab, "LogicalProject(A=[$0])")
    assert_columns_equal(out[0], expect(t, g["col1"], [1] * 7))
    out = engine.process_project(tab, "LogicalProject(C=[$2])")
    assert_columns_equal(out[0], expect(t, g["col3"], [1] * 7))
    out = engine.process_project(tab, "LogicalProject(A=[$0], C=[$2])")
    assert_columns_equal(out[0], expect(t, g["col1"]))
    assert_columns_equal(out[1], expect(t, g["col3"]))
    out = engine.process_project(tab, "LogicalProject(EXPR$0=[1])")
    assert_columns_equal(out[0], expect(T.INT32, [1] * 7))
    g5 = GOLD["project_gt3"]
    out = engine.process_project(tab, "LogicalProject(EXPR$0=[>($0, 3)])")
    assert_columns_equal(out[0], expect(T.BOOL8, g5["bool"] if t == T.BOOL8 else g5["other"]))
    g6 = GOLD["project_gt3_lt3"]
    out = engine.process_project(tab, "LogicalProject(EXPR$0=[>($0, 3)], EXPR$1=[<($2, 3)])")
    assert_columns_equal(out[0], expect(T.BOOL8, g6["bool_col1"] if t == T.BOOL8 else g6["other_col1"]))
    assert_columns_equal(out[1], expect(T.BOOL8, g6["bool_col3"] if t == T.BOOL8 else g6["other_col3"]))


# --------------------------------------------------- process_project.cpp:492-513
@pytest.mark.parametrize("t", [T.FLOAT32, T.FLOAT64])
def test_project_round(engine, t):
    g = GOLD["project_round"]
    tab = [column(t, g["input"])]
    out = engine.process_project(tab, "LogicalProject(EXPR$0=[ROUND($0)], EXPR$1=[ROUND($0, 2)], "
                                      "EXPR$2=[ROUND($0, 5)])")
    for k, key in enumerate(["round0", "round2", "round5"]):
        assert_columns_equal(out[k], expect(t, g[key]), ulps=0, what=key)


# --------------------------------------------------- filter_tests.cpp:23-172
@pytest.mark.parametrize("t", NUMERIC_TYPES)
def test_filter_empty_input(engine, t):
    out = engine.process_filter([HostColumn(t, np.zeros(0, np_dtype(t)))],
                                "LogicalFilter(condition=[<(+($0, $1), 0)])")
    assert out[0].size == 0 and out[0].type_id == t


@pytest.mark.parametrize("t", NUMERIC_TYPES)
def test_filter_empty_output(engine, t):
    r = np.arange(10)
    out = engine.process_filter([column(t, r), column(t, 2 * r)], "LogicalFilter(condition=[<(+($0, $1), 0)])")
    assert [c.size for c in out] == [0, 0]


@pytest.mark.parametrize("t", NUMERIC_TYPES)
def test_filter_mod(engine, t):
    r = np.arange(40)
    out = engine.process_filter([column(t, r), column(t, 2 * r)], "LogicalFilter(condition=[=(MOD(+($0, $1), 2), 0)])")
    n = 40 if t == T.BOOL8 else 20
    o = np.arange(n)
    assert_columns_equal(out[0], expect(t, 2 * o))
    assert_columns_equal(out[1], expect(t, 4 * o))


@pytest.mark.parametrize("t", NUMERIC_TYPES)
def test_filter_mod_with_nulls(engine, t):
    r = np.arange(40)
    valid = (r % 2) == 0
    out = engine.process_filter([column(t, r, valid), column(t, 2 * r, valid)],
                                "LogicalFilter(condition=[=(MOD(+($0, $1), 2), 0)])")
    o = np.arange(20)
    assert_columns_equal(out[0], expect(t, 2 * o, [1] * 20))
    assert_columns_equal(out[1], expect(t, 4 * o, [1] * 20))


# --------------------------------------------------- apply_filter.cpp:44-86
@pytest.mark.parametrize("t", NUMERIC_TYPES)
def test_apply_filter_with_nulls(engine, t):
    g = GOLD["apply_filter_with_null"]
    tab = [column(t, g["col1"], g["col1_valid"]), column(t, g["col3"], g["col3_valid"]),
           column(T.BOOL8, g["mask"], g["mask_valid"])]
    out = engine.process_filter(tab, "LogicalFilter(condition=[$2])")
    assert_columns_equal(out[0], expect(t, g["expect_col1"], g["expect_col1_valid"]))
    assert_columns_equal(out[1], expect(t, g["expect_col3"], g["expect_col3_valid"]))


# --------------------------------------------- kernel_projection_test.cpp:650-693
def test_large_literal(engine):
    tab = [column(T.INT16, [10, 40, 70, 5, 2, 10, 11]), column(T.INT32, [0] * 7),
           column(T.INT64, [1000, 4000, 7000, 500, 200, 100, 1100])]
    out = engine.process_project(tab, "LogicalProject(l_linenumber=[$0], l_comment=[$1], "
                                      "EXPR$2=[=($2, 100000000000)])")
    assert len(out) == 3 and out[2].size == 7 and out[2].type_id == T.BOOL8
    assert not out[2].values().any()
