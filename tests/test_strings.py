"""Strings on the evaluator's path, against the CPU oracle
(oracle/strings_ref.py) and the reference's own string-table tests:
the string pre-pass (LIKE, CHAR_LENGTH, comparisons with string literals and
between string columns, CASE with string results) evaluated on the GPU before
the plan kernel, and string output columns (copies, literals, and the
compaction of string columns by process_filter / filter_project)."""
from __future__ import annotations

import json
import os
import re

import numpy as np
import pytest

from blazingsql_gb300.types import HostColumn, TypeId as T, pack_validity
from oracle import strings_ref

from helpers import assert_columns_equal, assert_tables_equal

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.json")))
STRING_TABLES = {t["name"]: t for t in GOLD["string_tables"]}

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
def test_like_exhaustive_small_cases():
    """Every string of up to 5 characters over {a, b, newline} against LIKE
    patterns whose inner '%' must restart after a newline (the regular
    expression's search tries every start; '%' and '_' never cover a newline)."""
    import itertools
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    strs = [""] + ["".join(t) for k in range(1, 6) for t in itertools.product("ab\n", repeat=k)]
    pats = ["%a%a", "%b%_", "%%_%_", "%_%__", "%%b%a", "%a%_", "%_%a", "%_%b%", "a%b", "%a_b%", "_%", "%_",
            "a%", "%ab", "%a%b%a%", "__", "%b", "b%a%", "%", "",
            # middles over 15 bytes: the backtracking matcher instead of the automaton
            "%a%b%a%b%_%b%a%b%a", "a%a%a%a%a%a%a%a%a%", "%_%_%_%_%_%_%_%_%"]
    exprs = [f"LIKE($0, '{p}')" for p in pats]
    got = g.evaluate_expressions([DeviceColumn.from_strings(strs)], exprs)
    exp = strings_ref.evaluate_expressions([None], {0: strs}, exprs)
    _compare(got, exp, "LIKE small cases")


def test_like_automaton_host_matches_regex():
    """The byte automaton built for a LIKE pattern, walked on the host as the
    kernel walks it, against the reference's regular expression on random
    strings and patterns (newlines, multi-byte characters, '%' and '_')."""
    import ctypes as C
    import random
    from blazingsql_gb300 import _native as N
    lib = N.lib()
    rnd = random.Random(7)
    res, st = C.c_int32(), N.StatusInfo()
    checked = 0
    for _ in range(100_000):
        s = "".join(rnd.choice(["a", "b", "c", "\n", "é", "ß"]) for _ in range(rnd.randint(0, 10)))
        p = "".join(rnd.choice(["a", "b", "%", "_", "é"]) for _ in range(rnd.randint(0, 7)))
        b = s.encode()
        N.check(lib.gx_debug_like_automaton(p.encode(), b, len(b), C.byref(res), C.byref(st)), st)
        if res.value < 0:
            continue
        exp = re.search(strings_ref._py_regex(strings_ref.like_to_regex(p)), s) is not None
        assert bool(res.value) == exp, (s, p)
        checked += 1
    assert checked > 80_000  # the rest: empty or all-% patterns, which every string matches
    # a middle over 15 bytes is left to the backtracking matcher
    N.check(lib.gx_debug_like_automaton(b"%abcdefghijklmnopq%", b"x", 1, C.byref(res), C.byref(st)), st)
    assert res.value == -1


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


def _gold_table(t):
    """(host columns with None at string positions, {position: strings}) of a golden test's inputs."""
    cols, strings = [], {}
    for i, c in enumerate(t["inputs"]):
        valid = np.array(c["valid"], dtype=bool) if c["valid"] is not None else None
        if c["kind"] == "string":
            strings[i] = [v if valid is None or valid[k] else None for k, v in enumerate(c["values"])]
            cols.append(None)
        else:
            t, dt = GOLD_KINDS[c["kind"]]
            cols.append(HostColumn(t, np.array(c["values"], dtype=dt),
                                   pack_validity(valid) if valid is not None else None))
    return cols, strings


# element kinds of the reference's column wrappers
GOLD_KINDS = {"int32_t": (T.INT32, np.int32), "int": (T.INT32, np.int32), "bool": (T.BOOL8, np.uint8),
              "double": (T.FLOAT64, np.float64), "timestamp_s": (T.TIMESTAMP_SECONDS, np.int64),
              "timestamp_ns": (T.TIMESTAMP_NANOSECONDS, np.int64)}


def _gold_expected(c):
    valid = c["valid"]
    if c["kind"] == "string":
        return [v if valid is None or valid[k] else None for k, v in enumerate(c["values"])]
    t, dt = GOLD_KINDS[c["kind"]]
    return HostColumn(t, np.array(c["values"], dtype=dt),
                      pack_validity(np.array(valid, dtype=bool)) if valid is not None else None)


def _compare(got, exp, what):
    """got: HostColumn or list of strings (oracle) / NativeColumn (GPU); exp likewise."""
    assert len(got) == len(exp), what
    for i, (g, e) in enumerate(zip(got, exp)):
        if hasattr(g, "to_strings") and g.type_id == T.STRING:
            g = g.to_strings()
        elif hasattr(g, "to_host"):
            g = g.to_host()
        if isinstance(e, list):
            assert isinstance(g, list), f"{what} col {i}: expected strings"
            assert g == e, f"{what} col {i}: {g[:8]} vs {e[:8]}"
        else:
            assert_columns_equal(g, e, 0, f"{what} col {i}")


def _project_exprs(query):
    """The expressions of a LogicalProject(EXPR$0=[...], EXPR$1=[...]) query part."""
    body = re.fullmatch(r"LogicalProject\((.*)\)", query).group(1)
    out, depth, start = [], 0, None
    for i, ch in enumerate(body):
        if ch == "[":
            if depth == 0:
                start = i + 1
            depth += 1
        elif ch == "]":
            depth -= 1
            if depth == 0:
                out.append(body[start:i])
    return out


@pytest.mark.parametrize("name", sorted(STRING_TABLES))
def test_reference_string_tables_oracle(name):
    """The oracle reproduces the reference's string-table tests (filter_tests.cpp:174-215,
    process_project.cpp:286-485)."""
    t = STRING_TABLES[name]
    cols, strings = _gold_table(t)
    exp = [_gold_expected(c) for c in t["expected"]]
    if t["query"].startswith("LogicalFilter"):
        cond = re.search(r"condition=\[(.*)\]\)", t["query"]).group(1)
        got, rows = strings_ref.process_filter(cols, strings, cond)
        assert rows == len(t["expected"][0]["values"])
    else:
        got = strings_ref.evaluate_expressions(cols, strings, _project_exprs(t["query"]))
    _compare(got, exp, name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(STRING_TABLES))
def test_reference_string_tables_gpu(name):
    """The reference's string-table tests through process_filter / process_project."""
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    t = STRING_TABLES[name]
    cols, strings = _gold_table(t)
    dev = [DeviceColumn.from_strings(strings[i]) if c is None else DeviceColumn.from_host(c)
           for i, c in enumerate(cols)]
    exp = [_gold_expected(c) for c in t["expected"]]
    if t["query"].startswith("LogicalFilter"):
        got = g.process_filter(dev, t["query"])
    else:
        got, _ = g.process_project(dev, t["query"])
    _compare(got, exp, name)


def _mixed_table(rng, n):
    s0 = _strings(rng, n)
    s3 = _strings(rng, n, 0.3)
    x1 = HostColumn(T.INT64, rng.integers(-50, 50, n).astype(np.int64))
    v2 = rng.random(n) > 0.1
    x2 = HostColumn(T.FLOAT64, rng.normal(0, 10, n), pack_validity(v2))
    return [None, x1, x2, None], {0: s0, 3: s3}


def _device(cols, strings):
    from blazingsql_gb300.api import DeviceColumn
    return [DeviceColumn.from_strings(strings[i]) if c is None else DeviceColumn.from_host(c)
            for i, c in enumerate(cols)]


STRING_EXPRS = [
    "$0", "$3", "'lit'", "$1",
    "CASE(>($1, 0), $0, 'neg')", "CASE(>($1, 0), 'pos', $3)", "CASE(>($1, 0), $0, $3)",
    "CASE(IS NULL($2), null, $0)", "CASE(<($2, 0.0), $3, null)",
    "CASE(>($1, 20), 'big', <($1, -20), $0, =($1, 0), 'zero', $3)",
    "CASE(LIKE($0, '%a%'), $3, 'no a')",
    "=(CASE(>($1, 0), $0, 'x'), 'x')",
    "CHAR_LENGTH(CASE(>($1, 0), $0, 'éé'))",
    "=($0, $3)", "<($0, $3)", ">=($3, $0)", "<>($0, $3)",
    "CASE(>($1, 0), +($1, 1), -($1, 1))",
]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 37, 4099, 100_003])
def test_string_outputs_match_oracle(n):
    """String outputs (copies, literals, CASE with string results) and
    column-to-column string comparisons."""
    import blazingsql_gb300 as g
    rng = np.random.default_rng(100 + n)
    cols, strings = _mixed_table(rng, n)
    got = g.evaluate_expressions(_device(cols, strings), STRING_EXPRS)
    exp = strings_ref.evaluate_expressions(cols, strings, STRING_EXPRS)
    _compare(got, exp, f"string outputs n={n}")


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 37, 4099, 100_003])
def test_filter_compacts_string_columns(n):
    """process_filter keeps every column, string columns included, in order."""
    import blazingsql_gb300 as g
    rng = np.random.default_rng(200 + n)
    cols, strings = _mixed_table(rng, n)
    dev = _device(cols, strings)
    for cond in ["AND(>($1, 0), LIKE($0, '%b%'))", ">($3, 'b')", "OR(IS NULL($2), =($0, $3))", "<($1, 100)",
                 "<($1, -100)"]:
        got = g.process_filter(dev, f"LogicalFilter(condition=[{cond}])")
        exp, rows = strings_ref.process_filter(cols, strings, cond)
        assert got[0].size == rows
        _compare(got, exp, f"process_filter {cond} n={n}")


@pytest.mark.gpu
def test_filter_project_string_outputs():
    import blazingsql_gb300 as g
    rng = np.random.default_rng(7)
    n = 50_001
    cols, strings = _mixed_table(rng, n)
    cond = "AND(>($1, -10), NOT(LIKE($3, 'a%')))"
    exprs = ["$3", "*($2, 2.0)", "CASE(>($1, 0), $0, 'neg')", "'k'", "$0", "CHAR_LENGTH($0)"]
    got = g.filter_project(_device(cols, strings), cond, exprs)
    exp, rows = strings_ref.filter_project(cols, strings, cond, exprs)
    assert got[0].size == rows
    _compare(got, exp, "filter_project with string outputs")


@pytest.mark.gpu
def test_string_column_views_with_offset():
    """Views starting inside a string column (offset > 0): offsets and masks
    are read from the view's first row."""
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    rng = np.random.default_rng(9)
    n, k = 5000, 77
    full = _strings(rng, n + k)
    fx = HostColumn(T.INT64, rng.integers(-50, 50, n + k).astype(np.int64))
    sc = DeviceColumn.from_strings(full)
    xc = DeviceColumn.from_host(fx)
    dev = [DeviceColumn(sc.type_id, sc.data, sc.mask, k, n, sc.str_offsets),
           DeviceColumn(xc.type_id, xc.data, xc.mask, k, n)]
    cols = [None, HostColumn(T.INT64, fx.data[k:].copy())]
    strings = {0: full[k:]}
    exprs = ["$0", "CASE(>($1, 0), $0, 'z')", "LIKE($0, '%a%')"]
    _compare(g.evaluate_expressions(dev, exprs), strings_ref.evaluate_expressions(cols, strings, exprs), "offset view")
    got = g.process_filter(dev, "LogicalFilter(condition=[>($1, 0)])")
    exp, _ = strings_ref.process_filter(cols, strings, ">($1, 0)")
    _compare(got, exp, "offset view filter")


@pytest.mark.gpu
def test_string_empty_inputs():
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    dev = [DeviceColumn.from_strings([]), DeviceColumn.from_host(HostColumn(T.INT32, np.zeros(0, np.int32)))]
    out = g.process_filter(dev, "LogicalFilter(condition=[=($0, 'a')])")
    assert [c.size for c in out] == [0, 0] and out[0].to_strings() == []
    dev = [DeviceColumn.from_strings(["", None, ""]), DeviceColumn.from_host(HostColumn(T.INT32, np.arange(3, dtype=np.int32)))]
    out = g.evaluate_expressions(dev, ["$0", "CASE(>($1, 0), $0, '')"])
    assert out[0].to_strings() == ["", None, ""]
    assert out[1].to_strings() == ["", None, ""]
    out = g.process_filter(dev, "LogicalFilter(condition=[<($1, 0)])")
    assert out[0].to_strings() == [] and out[1].size == 0
    # string functions made after a filter that keeps no row, and over an empty table
    exprs = ["UPPER($0)", "CONCAT($0, '-', CAST($1):VARCHAR)", "SUBSTRING($0, $1)", "REGEXP_REPLACE($0, 'a', 'b')"]
    out = g.filter_project(dev, "<($1, 0)", exprs)
    assert [c.to_strings() for c in out] == [[]] * 4
    empty = [DeviceColumn.from_strings([]), DeviceColumn.from_host(HostColumn(T.INT32, np.zeros(0, np.int32)))]
    out = g.filter_project(empty, ">($1, 0)", exprs)
    assert [c.to_strings() for c in out] == [[]] * 4
    out = g.filter_project(dev, ">=($1, 1)", exprs)
    assert [c.to_strings() for c in out] == [[None, ""], [None, "-2"], [None, ""], [None, ""]]


def _function_table(rng, n):
    """String, numeric and temporal columns for the string functions."""
    s0 = _strings(rng, n)
    s3 = [None if v is None else " " * int(rng.integers(0, 3)) + v + " " * int(rng.integers(0, 3))
          for v in _strings(rng, n, 0.2)]
    nums = ["-12", "+7", "300", "12ab", "", "abc", "99999999999", "-0", "2147483648", "-9223372036854775808"]
    s9 = [None if rng.random() < 0.1 else nums[int(rng.integers(0, len(nums)))] for _ in range(n)]
    days = rng.integers(-1000, 20000, n)
    s10 = [None if rng.random() < 0.1 else str(np.datetime64("1970-01-01") + np.timedelta64(int(d), "D")) for d in days]
    secs = rng.integers(0, 2_000_000_000, n)
    s11 = [None if rng.random() < 0.1 else str(np.datetime64(int(x), "s")).replace("T", " ") for x in secs]
    ascii_alpha = list("abcXYZ 09-_.")
    s12 = [None if rng.random() < 0.1 else "".join(rng.choice(ascii_alpha, int(rng.integers(0, 9))))
           for _ in range(n)]
    v = rng.random(n) > 0.1
    cols = [None,
            HostColumn(T.INT64, np.concatenate([[np.iinfo(np.int64).min], rng.integers(-10**12, 10**12, n - 1)])[:n]
                       .astype(np.int64), pack_validity(v)),
            HostColumn(T.FLOAT64, rng.normal(0, 10, n)),
            None,
            HostColumn(T.BOOL8, (rng.random(n) > 0.5).astype(np.uint8), pack_validity(rng.random(n) > 0.1)),
            HostColumn(T.INT32, rng.integers(-2**31, 2**31 - 1, n).astype(np.int32)),
            HostColumn(T.TIMESTAMP_DAYS, rng.integers(-5000, 40000, n).astype(np.int32)),
            HostColumn(T.TIMESTAMP_SECONDS, rng.integers(0, 4_000_000_000, n).astype(np.int64)),
            HostColumn(T.TIMESTAMP_MILLISECONDS, rng.integers(-10**12, 4 * 10**12, n).astype(np.int64)),
            None, None, None, None, None]
    s13 = [None if v is None else f"{v[8:10]}/{v[5:7]}/{v[:4]}" for v in s10]  # day/month/year
    # floating-point texts: exact short decimals, full round-trip reprs, exponents,
    # specials and malformed ones
    texts = ["1.5", "-2e3", "1e400", ".5", "  1", "abc", "1.2.3", "12345678901234567890123", "NaN", "-Inf",
             "0.1", "3.24e-05", "+7.", "1E+2", "-0", "", "999999.001", "0.45435436", "1e-320", "5e-324x"]
    s14 = [None if rng.random() < 0.1 else
           (texts[int(rng.integers(0, len(texts)))] if rng.random() < 0.4 else
            repr(float(rng.normal(0, 10) * 10.0 ** int(rng.integers(-30, 30)))) if rng.random() < 0.5 else
            f"{rng.uniform(-1000, 1000):.{int(rng.integers(0, 7))}f}") for _ in range(n)]
    # doubles over the whole exponent range, with the rounding edges of the format
    wide = np.sign(rng.normal(size=n)) * 10.0 ** rng.uniform(-325, 308.2, n)
    edges = [0.0, -0.0, np.inf, -np.inf, np.nan, 1e9, 1e-4, 9.9999e-5, 999999999.9999999, 0.99999999995,
             9.9999999999e20, 123456789.0, 1234567891.0, 5e-324, 1.7976931348623157e308, 0.1 + 0.2]
    k = min(len(edges), n)
    wide[:k] = edges[:k]
    cols += [None,
             HostColumn(T.FLOAT32, rng.normal(0, 1000, n).astype(np.float32), pack_validity(rng.random(n) > 0.1)),
             HostColumn(T.FLOAT64, wide),
             HostColumn(T.INT32, rng.integers(-3, 10, n).astype(np.int32), pack_validity(rng.random(n) > 0.15))]
    # non-ASCII text for the case mappings: one-to-many (ß, ŉ, ﬀ, ΐ), İ, title-case
    # digraphs, final sigma, Cyrillic, Deseret (4-byte), combining marks, digits
    uni = list("aßŉﬀΐİǅǆǄΣσςЖжẞ𐐨𐐀ÀàÉé ́-1٣_xZ") + ["😀", "ǰ"]
    s18 = [None if rng.random() < 0.1 else "".join(rng.choice(uni, int(rng.integers(0, 9)))) for _ in range(n)]
    cols.append(None)
    return cols, {0: s0, 3: s3, 9: s9, 10: s10, 11: s11, 12: s12, 13: s13, 14: s14, 18: s18}


FUNCTION_EXPRS = [
    "SUBSTRING($0, 2, 3)", "SUBSTRING($0, 0)", "SUBSTRING($0, 3)", "SUBSTRING($0, -1, 2)", "SUBSTRING($0, 2, 0)",
    "LEFT($0, 2)", "LEFT($0, 0)", "RIGHT($0, 2)", "RIGHT($0, 0)", "RIGHT($0, 10)", "REVERSE($0)",
    "TRIM(FLAG(BOTH), ' ', $3)", "TRIM(FLAG(LEADING), 'ab', $0)", "TRIM(FLAG(TRAILING), 'é ', $3)",
    "REPLACE($0, 'ab', 'X')", "REPLACE($3, ' ', '')",
    "CONCAT($0, $3)", "||($0, '-')", "CONCAT('<', $0, '|', $3, '>')",
    "CONCAT(CONCAT($0, 'x'), ||($3, $12), $0)", "CONCAT($0, '1', $3, '2', $12, '3', $0, '4', $3, '5')",
    "CONCAT($0, '#', CAST($5):VARCHAR, CAST($6):VARCHAR, CAST($4):VARCHAR)", "||(CAST($1):VARCHAR, $3)",
    "CAST($1):VARCHAR", "CAST($4):VARCHAR", "CAST($5):VARCHAR", "CAST($6):VARCHAR", "CAST($7):VARCHAR",
    "CAST($8):VARCHAR", "CAST(+($1, 7)):VARCHAR", "CAST($0):VARCHAR", "CAST(5):VARCHAR",
    "CAST($9):INTEGER", "CAST($9):BIGINT", "CAST($9):TINYINT", "CAST($9):SMALLINT", "CAST($10):DATE",
    "CAST($11):TIMESTAMP", "CAST($11):TIMESTAMP_SECONDS",
    "=(SUBSTRING($0, 1, 2), 'ab')", "CHAR_LENGTH(CONCAT($0, $3))", "+(CAST($9):INTEGER, 1)",
    "UPPER($12)", "LOWER($12)", "INITCAP($12)", "CASE(>($5, 0), UPPER($12), REVERSE($0))",
    "TO_DATE($10, '%Y-%m-%d')", "TO_TIMESTAMP($11, '%Y-%m-%d %H:%M:%S')", "TO_DATE($13, '%d/%m/%Y')",
    "TO_TIMESTAMP($13, '%d/%m/%Y')", "TO_DATE($11, '%Y%%%m%d')",
    "CAST($2):VARCHAR", "CAST($15):VARCHAR", "CAST($16):VARCHAR", "CONCAT($0, '=', CAST($16):VARCHAR)",
    "CAST($14):DOUBLE", "CAST($14):FLOAT", "CAST(CAST($16):VARCHAR):DOUBLE",
    "SUBSTRING($0, $17)", "SUBSTRING($0, $17, 2)", "SUBSTRING($0, 2, $17)", "SUBSTRING($0, $17, CHAR_LENGTH($3))",
    "SUBSTRING($0, 2, -(CHAR_LENGTH($0), 2))", "SUBSTRING($3, +($17, 1), $17)",
    "UPPER($18)", "LOWER($18)", "INITCAP($18)", "CHAR_LENGTH(UPPER($18))", "UPPER($0)", "INITCAP($3)",
]


def test_string_functions_oracle_rules():
    """Slices by characters (cudf slice_strings), formatting and parsing rules of the oracle."""
    assert strings_ref._slice("héllo", 1, 4, 1) == "éll"
    assert strings_ref._slice("abc", -2, None, 1) == "bc"          # RIGHT($0, 2)
    assert strings_ref._slice("abc", 0, 0, 1) == ""                # RIGHT($0, 0)
    assert strings_ref._slice("aé", None, None, -1) == "éa"        # REVERSE, by characters
    assert strings_ref.parse_value(T.INT8, "300") == 44            # wrapped to the type
    assert strings_ref.parse_value(T.INT32, "-12ab") == -12        # digits up to the first other character
    assert strings_ref.parse_value(T.TIMESTAMP_DAYS, "1996-12-31") == 9861
    assert strings_ref.format_value(T.TIMESTAMP_SECONDS, 851990400 + 3661) == "1996-12-31 01:01:01"
    assert strings_ref.format_value(T.TIMESTAMP_MILLISECONDS, -1) == "1969-12-31 23:59:59"
    assert strings_ref.parse_value(T.TIMESTAMP_DAYS, "31/12/1996", "%d/%m/%Y") == 9861
    assert strings_ref.parse_value(T.TIMESTAMP_DAYS, "1996-12", "%Y-%m-%d") == strings_ref._days_from_civil(1996, 12, 0)
    assert strings_ref.format_value(T.FLOAT64, 1e9) == "1.0e+09"              # from 1e9: scientific
    assert strings_ref.format_value(T.FLOAT64, 1234567891.0) == "1.234567891e+09"
    assert strings_ref.format_value(T.FLOAT64, 0.1 + 0.2) == "0.3"            # 9 significant digits
    assert strings_ref.format_value(T.FLOAT64, -0.0) == "-0.0"
    assert strings_ref.format_value(T.FLOAT64, float("inf")) == "Inf"
    assert strings_ref.parse_value(T.FLOAT64, "-2e3") == -2000.0
    assert strings_ref.parse_value(T.FLOAT64, "1.2.3") == 1.2                 # up to the second point
    assert strings_ref._slice_cols("abcdef", -2, 3) == "abc"                   # start clamped at 0
    assert strings_ref._slice_cols("abcdef", 2, -1) == "cdef"                  # a negative stop: the end
    assert strings_ref._slice_cols("abc", 2, 1) == ""
    texts, ops = strings_ref.rewrite(["CONCAT($0, '-', $1)"], [0, 1], 2)
    assert texts == ["$3"] and [o[0] for o in ops] == ["CONCAT", "CONCAT"]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 37, 4099, 60_001])
def test_string_functions_match_oracle(n):
    """SUBSTRING / LEFT / RIGHT / REVERSE / TRIM / REPLACE / CONCAT / UPPER /
    LOWER / INITCAP and CASTs to and from VARCHAR against the oracle."""
    import blazingsql_gb300 as g
    rng = np.random.default_rng(300 + n)
    cols, strings = _function_table(rng, n)
    got = g.evaluate_expressions(_device(cols, strings), FUNCTION_EXPRS)
    exp = strings_ref.evaluate_expressions(cols, strings, FUNCTION_EXPRS)
    _compare(got, exp, f"string functions n={n}")


@pytest.mark.gpu
def test_string_functions_in_filters():
    import blazingsql_gb300 as g
    rng = np.random.default_rng(11)
    n = 30_011
    cols, strings = _function_table(rng, n)
    dev = _device(cols, strings)
    cond = "AND(=(LEFT($12, 1), 'a'), >(CAST($9):INTEGER, 0))"
    # string functions read only as outputs are made after the filter, for
    # the kept rows alone (through the row map); LEFT($12, 1) is read by the
    # condition and made before it
    exprs = ["CONCAT($0, '/', CAST($5):VARCHAR)", "$12", "CAST($10):DATE", "REVERSE($3)",
             "SUBSTRING($0, $17, CHAR_LENGTH($3))", "REGEXP_REPLACE($0, '[ab]+', '<\\0>')", "UPPER($18)",
             "CAST($16):VARCHAR", "CAST(+($1, 7)):VARCHAR", "LEFT($12, 1)", "INITCAP($12)", "INITCAP($12)",
             "CHAR_LENGTH(TRIM(FLAG(BOTH), ' ', $3))"]
    got = g.filter_project(dev, cond, exprs)
    exp, rows = strings_ref.filter_project(cols, strings, cond, exprs)
    assert got[0].size == rows
    _compare(got, exp, "string functions under a filter")


@pytest.mark.gpu
def test_string_function_errors():
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300.api import DeviceColumn
    dev = [DeviceColumn.from_strings(["é", "b"]), DeviceColumn.from_host(HostColumn(T.FLOAT64, np.arange(2.0)))]
    with pytest.raises(N.GxError, match="integer column"):
        g.evaluate_expressions(dev, ["SUBSTRING($0, $1)"])  # LogicalProject.cpp:252
    with pytest.raises(N.GxError, match="between literals"):
        g.evaluate_expressions(dev, ["CONCAT('a', 'b')"])
    with pytest.raises(N.GxError, match="between literals"):
        g.evaluate_expressions(dev, ["CONCAT('a', 'b', $0)"])  # its innermost pair
    with pytest.raises(N.GxError, match="without"):
        g.evaluate_expressions(dev, ["TO_DATE($0, '%Y-%m')"])
    with pytest.raises(N.GxError, match="specifier"):
        g.evaluate_expressions(dev, ["TO_TIMESTAMP($0, '%Y-%m-%d %I')"])


def test_case_tables_match_the_oracles_unicode():
    """The device's case tables come from the same Unicode version as the
    oracle's str.upper / str.lower / str.isalpha."""
    import unicodedata
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "blazingsql_gb300", "csrc",
                        "case_tables.inc")
    head = open(path).read(400)
    m = re.search(r'GX_CASE_UNICODE_VERSION "([0-9.]+)"', head)
    if m.group(1) != unicodedata.unidata_version:
        pytest.skip(f"this Python's Unicode {unicodedata.unidata_version} is not the tables' {m.group(1)}")
    # the committed tables are what the generator writes from this Unicode version
    import importlib.util
    import io
    spec = importlib.util.spec_from_file_location("gen_case_tables", os.path.join(os.path.dirname(path),
                                                                                  "gen_case_tables.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    buf = io.StringIO()
    gen.main(buf)
    body = lambda t: "\n".join(l for l in t.splitlines() if not l.startswith("//"))  # noqa: E731
    assert body(buf.getvalue()) == body(open(path).read())
    assert strings_ref._upper("straße ŉ") == "STRASSE ʼN"
    assert strings_ref._lower("ΣΑΣ") == "σασ"                  # per code point: no final sigma
    assert strings_ref._initcap("ǆemal élan-x1y") == "Ǆemal Élan-X1Y"


def test_string_rewrite_oracle_rules():
    """Children-first rewriting: a string CASE becomes a column that an
    enclosing comparison then reads; CASE pairs fold from the innermost."""
    texts, ops = strings_ref.rewrite(["=(CASE(=(MOD($0, 2), 0), $1, 'LOL'), 'LOL')"], [1], 2)
    assert texts == ["$3"]
    assert ops[0][0] == "CASE" and ops[1] == ("EQ", 2, "LOL")
    texts, ops = strings_ref.rewrite(["CASE(>($0, 1), 'a', >($0, 0), $1, 'c')"], [1], 2)
    assert texts == ["$3"] and [o[0] for o in ops] == ["CASE", "CASE"]
    assert ops[1][2] == ("lit", "a") and ops[1][3] == ("col", 2)
    with pytest.raises(ValueError):
        strings_ref.rewrite(["+(CASE(>($0, 1), $1, 'a'), 1)"], [1], 2)


@pytest.mark.gpu
def test_string_errors():
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300.api import DeviceColumn
    dev = [DeviceColumn.from_strings(["a", "b"]), DeviceColumn.from_host(HostColumn(T.INT64, np.arange(2)))]
    with pytest.raises(N.GxError, match="string column"):
        g.evaluate_expressions(dev, ["+($0, 1)"])            # a string column in arithmetic
    with pytest.raises(N.GxError, match="regular-expression"):
        g.evaluate_expressions(dev, ["LIKE($0, 'a.b')"])     # the reference's regex semantics are not restated
    with pytest.raises(N.GxError, match="condition expression literals"):
        g.evaluate_expressions(dev, ["CASE(true, $0, 'x')"])  # LogicalProject.cpp:627
    with pytest.raises(N.GxError, match="condition is a string"):
        g.process_filter(dev, "LogicalFilter(condition=[$0])")
