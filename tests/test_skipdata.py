"""Skip-data (row-group pruning) predicate: the rewrite rules of
ral::skip_data against the reference's own test vectors
(engine/tests/skipdata/expression_tree_test.cpp, extracted into
tests/golden/reference_vectors.json), for the library (C ABI, no GPU) and the
CPU oracle; on the GPU, the row groups kept from a statistics table against
the oracle."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from blazingsql_gb300.types import HostColumn, TypeId as T
from oracle import skipdata_ref

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.json")))
CASES = GOLD["skip_data_rewrite"]["cases"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_rewrite_matches_reference_tests(case):
    text, pre = skipdata_ref.rewrite(case["input"], case["dropped"])
    assert pre == case["expected"], case["source"]
    assert (text == "") == (case["expected"] == "NONE")


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_library_rewrite_matches_reference_tests(case):
    import blazingsql_gb300 as g
    pre, usable = g.api.skip_data_rewrite(case["input"], case["dropped"], prefix_form=True)
    assert pre == case["expected"], case["source"]
    assert usable == (case["expected"] != "NONE")
    text, _ = g.api.skip_data_rewrite(case["input"], case["dropped"])
    assert text == skipdata_ref.rewrite(case["input"], case["dropped"])[0]


def _metadata(rng, groups):
    """Row-group statistics of a 3-column table: per group, sorted random
    bounds; column 1 has no statistics."""
    names = ["c_custkey", "c_nationkey", "c_acctbal"]
    md = {}
    lo0 = rng.integers(0, 30000, groups)
    md["min_0_c_custkey"] = HostColumn(T.INT64, lo0.astype(np.int64))
    md["max_0_c_custkey"] = HostColumn(T.INT64, (lo0 + rng.integers(0, 2000, groups)).astype(np.int64))
    lo2 = rng.normal(0, 500, groups)
    md["min_2_c_acctbal"] = HostColumn(T.FLOAT64, lo2)
    md["max_2_c_acctbal"] = HostColumn(T.FLOAT64, lo2 + np.abs(rng.normal(0, 300, groups)))
    ids = (np.repeat(np.arange(4), (groups + 3) // 4)[:groups].astype(np.int32),
           np.arange(groups, dtype=np.int32))
    return md, names, ids


@pytest.mark.gpu
@pytest.mark.parametrize("scan", [
    "BindableTableScan(table=[[main, customer]], filters=[[OR(AND(<($0, 15000), =($1, 5)), >=($2, 100.5))]], "
    "projects=[[0, 1, 2]], aliases=[[a, b, c]])",
    "BindableTableScan(table=[[main, customer]], filters=[[AND(>($0, 20000), <=($1, 10.0))]], "
    "projects=[[0, 2]], aliases=[[a, c]])",
    "BindableTableScan(table=[[main, customer]], filters=[[=(+($0, $0), 30000)]], projects=[[0]], aliases=[[a]])",
    "BindableTableScan(table=[[main, customer]], filters=[[OR(IS NOT NULL($0), =($1, 5))]], "
    "projects=[[0, 1]], aliases=[[a, b]])",
])
def test_row_groups_match_oracle(scan):
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    rng = np.random.default_rng(9)
    groups = 5000
    md, names, ids = _metadata(rng, groups)
    mnames = list(md) + ["file_handle_index", "row_group_index"]
    mcols = list(md.values()) + [HostColumn(T.INT32, ids[0]), HostColumn(T.INT32, ids[1])]
    got, rows = g.api.skip_data_filter([DeviceColumn.from_host(c) for c in mcols], mnames, names, scan)
    filt = scan.split("filters=[[")[1].split("]], projects")[0]
    proj = [int(x) for x in scan.split("projects=[[")[1].split("]]")[0].split(",")]
    exp = skipdata_ref.row_groups(md, names, filt, proj, ids)
    if exp is None:
        assert got is None
        return
    h = [c.to_host() for c in got]
    assert rows == len(exp[0])
    assert list(h[0].data) == exp[0] and list(h[1].data) == exp[1]
