"""String pre-pass: LIKE, CHAR_LENGTH and comparisons with string literals
over cudf-layout string columns, evaluated on the GPU before the plan kernel,
against the CPU oracle (oracle/strings_ref.py), which follows the reference's
LIKE-to-regex translation and string_view comparisons."""
from __future__ import annotations

import numpy as np
import pytest

from blazingsql_gb300.types import HostColumn, TypeId as T
from oracle import strings_ref

from helpers import assert_tables_equal

ALPHA = ["a", "b", "c", "é", "ab", "PROMO", "\n", "%", "x_y", "ß"]


def _strings(rng, n, null_frac=0.1):
    out = []
    for _ in range(n):
        if rng.random() < null_frac:
            out.append(None)
        else:
            out.append("".join(rng.choice(ALPHA, rng.integers(0, 6))))
    return out


def test_like_regex_translation():
    """like_expression_to_regex_str's anchors and wildcards (LogicalProject.cpp:31-47)."""
    assert strings_ref.like_to_regex("PROMO%") == "^PROMO(?:.*?)"
    assert strings_ref.like_to_regex("%ab_c") == "(?:.*?)ab(?:.)c$"
    assert strings_ref.like_to_regex("") == ""
    col = ["PROMO1", "xPROMO", None, "", "a\nb", "a", "é"]
    c = strings_ref.evaluate_op(("LIKE", 0, "PROMO%"), col)
    assert list(c.data) == [1, 0, 0, 0, 0, 0, 0]
    assert list(strings_ref.evaluate_op(("LIKE", 0, "a_b"), col).data) == [0, 0, 0, 0, 0, 0, 0]  # '_' skips no newline
    assert list(strings_ref.evaluate_op(("LIKE", 0, "_"), col).data) == [0, 0, 0, 0, 0, 1, 1]   # one character, UTF-8
    assert list(strings_ref.evaluate_op(("LIKE", 0, ""), col).data) == [1, 1, 0, 1, 1, 1, 1]    # empty regex matches


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 33, 5000, 100_003])
def test_string_operators_match_oracle(n):
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    rng = np.random.default_rng(n)
    s0 = _strings(rng, n)
    x1 = HostColumn(T.INT64, rng.integers(-50, 50, n).astype(np.int64))
    exprs = ["LIKE($0, 'PROMO%')", "LIKE($0, '%ab_c%')", "LIKE($0, 'a%b')", "LIKE($0, '_')", "LIKE($0, '')",
             "LIKE($0, '%é%')", "CHAR_LENGTH($0)", "=($0, 'ab')", "<>($0, 'ab')", "<('c', $0)", ">=($0, 'b')",
             "AND(LIKE($0, '%a%'), >($1, 0))", "+(CHAR_LENGTH($0), $1)", "NOT(LIKE($0, '%b%'))"]
    dev = [DeviceColumn.from_strings(s0), DeviceColumn.from_host(x1)]
    got = [c.to_host() for c in g.evaluate_expressions(dev, exprs)]
    exp = strings_ref.evaluate_expressions([None, x1], {0: s0}, exprs)
    assert_tables_equal(got, exp, what=f"string operators n={n}")


@pytest.mark.gpu
def test_filter_with_like_matches_oracle():
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    rng = np.random.default_rng(4)
    n = 70_001
    s0 = _strings(rng, n)
    x1 = HostColumn(T.INT64, rng.integers(-50, 50, n).astype(np.int64))
    x2 = HostColumn(T.FLOAT64, rng.normal(0, 10, n))
    cond = "OR(AND(LIKE($0, 'PROMO%'), >($1, 10)), =($0, 'ab'))"
    exprs = ["$1", "*($2, 2.0)", "CHAR_LENGTH($0)"]
    dev = [DeviceColumn.from_strings(s0), DeviceColumn.from_host(x1), DeviceColumn.from_host(x2)]
    got = [c.to_host() for c in g.filter_project(dev, cond, exprs)]
    exp, rows = strings_ref.filter_project([None, x1, x2], {0: s0}, cond, exprs)
    assert len(got[0].data) == rows
    assert_tables_equal(got, exp, what="filter with LIKE")


@pytest.mark.gpu
def test_string_errors():
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300.api import DeviceColumn
    dev = [DeviceColumn.from_strings(["a", "b"]), DeviceColumn.from_host(HostColumn(T.INT64, np.arange(2)))]
    with pytest.raises(N.GxError, match="string column"):
        g.evaluate_expressions(dev, ["$0"])                   # a string output is not produced
    with pytest.raises(N.GxError, match="regular-expression"):
        g.evaluate_expressions(dev, ["LIKE($0, 'a.b')"])     # the reference's regex semantics are not restated
