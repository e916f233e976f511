"""preprocess_expression's text rewrites (engine/src/parser/expression_utils.cpp:1624-1632):
pinned by the reference's own test vectors where it has them
(engine/tests/parser/expression_utils_test.cpp: convert_ms_to_ns_units,
reinterpret_timestamp), and restating its code for apply_interval_conversion
(:1425-1460) and get_current_date_or_timestamp (:1494-1518), which its tests do
not cover."""
import json
import os

import numpy as np
import pytest

import blazingsql_gb300 as g
from blazingsql_gb300.types import HostColumn, TypeId as T
from tests.helpers import GpuEngine, OracleEngine, assert_tables_equal

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.json")))
STAGE = {"convert_ms_to_ns_units": 4, "reinterpret_timestamp": 8}


@pytest.mark.parametrize("case", GOLD["preprocess_rewrites"], ids=lambda c: c["name"])
def test_reference_rewrite_vectors(case):
    schema = [int(getattr(T, name)) for name in case["schema"]]
    assert g.api.preprocess(case["input"], schema, STAGE[case["function"]]) == case["expected"], case["source"]


@pytest.mark.parametrize("unit, expected", [
    (T.DURATION_SECONDS, "+($0, 86400:INTERVAL DAY)"),
    (T.DURATION_MILLISECONDS, "+($0, 86400000:INTERVAL DAY)"),
    (T.DURATION_MICROSECONDS, "+($0, 86400000000:INTERVAL DAY)"),
    (T.DURATION_NANOSECONDS, "+($0, 86400000000000:INTERVAL DAY)"),
])
def test_interval_units_follow_the_column(unit, expected):
    # Calcite gives intervals in milliseconds; the column's unit decides the scale
    assert g.api.preprocess("+($0, 86400000:INTERVAL DAY)", [unit, T.INT32], 16) == expected
    assert g.api.preprocess("-($0, 86400000:INTERVAL DAY)", [unit], 16) == expected.replace("+", "-", 1)


def test_interval_rewrites_every_occurrence_and_literals():
    two = "+($0, CASE($1, 60000:INTERVAL MINUTE, 3600000:INTERVAL HOUR))"
    assert g.api.preprocess(two, [T.DURATION_SECONDS, T.BOOL8], 16) == \
        "+($0, CASE($1, 60:INTERVAL MINUTE, 3600:INTERVAL HOUR))"
    assert g.api.preprocess("1000:INTERVAL SECOND", [T.INT32], 16) == "1:INTERVAL SECOND"
    assert g.api.preprocess("+($0, 1000:INTERVAL SECOND)", [], 16) == "+($0, 1000:INTERVAL SECOND)"  # no schema


def test_current_date_and_timestamp():
    g.api.set_current_timestamp("2021-05-14 10:11:12.345678")
    try:
        assert g.api.preprocess(">($0, CURRENT_DATE)", [T.TIMESTAMP_DAYS]) == ">($0, 2021-05-14)"
        assert g.api.preprocess("<($0, CURRENT_TIMESTAMP)", []) == "<($0, 2021-05-14 10:11:12.345)"
        assert g.api.preprocess("<($0, CURRENT_TIME)", []) == "<($0, 2021-05-14 10:11:12.345)"
        # both present: only CURRENT_DATE is replaced (the reference's rule)
        assert g.api.preprocess("AND(>($0, CURRENT_DATE), <($1, CURRENT_TIMESTAMP))", []) == \
            "AND(>($0, 2021-05-14), <($1, CURRENT_TIMESTAMP))"
        assert g.api.preprocess("=($0, CURRENT_DATE)", [], 31 & ~2) == "=($0, CURRENT_DATE)"  # stage off
    finally:
        g.api.set_current_timestamp(None)
    with pytest.raises(g.GxError) as ei:
        g.api.preprocess(">($0, CURRENT_DATE)", [T.TIMESTAMP_DAYS])
    assert ei.value.code == g._native.GX_ERR_UNSUPPORTED
    for bad in ("2021-05-14", "2021/05/14 10:11:12", "2021-05-14T10:11:12", "x"):
        with pytest.raises(g.GxError):
            g.api.set_current_timestamp(bad)


@pytest.mark.gpu
def test_current_date_evaluates_as_the_literal():
    rng = np.random.default_rng(3)
    n = 5000
    days = rng.integers(18700, 18800, n).astype(np.int32)  # around 2021-05-14 (day 18761)
    ms = rng.integers(1620950000000, 1621050000000, n, dtype=np.int64)
    cols = [HostColumn(T.TIMESTAMP_DAYS, days), HostColumn(T.TIMESTAMP_MILLISECONDS, ms)]
    g.api.set_current_timestamp("2021-05-14 10:11:12.345678")
    try:
        # process_project preprocesses its expressions (evaluate_expressions takes them preprocessed)
        got = GpuEngine().process_project(
            cols, "LogicalProject(d=[>=($0, CURRENT_DATE)], t=[<($1, CURRENT_TIMESTAMP)])")
    finally:
        g.api.set_current_timestamp(None)
    exp = OracleEngine(2).evaluate_expressions(cols, [">=($0, 2021-05-14)", "<($1, 2021-05-14 10:11:12.345)"])
    assert_tables_equal(got, exp, what="CURRENT_DATE / CURRENT_TIMESTAMP")
    assert 0 < int(got[0].values().sum()) < n and 0 < int(got[1].values().sum()) < n
