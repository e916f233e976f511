"""C-ABI boundary checks that need no GPU: the library loads, exports every
symbol include/gx_eval.h declares, reports parse / type / unsupported errors
through status codes, and its generated plan kernels compile for sm_103a."""
import ctypes as C
import os
import re

import pytest

import blazingsql_gb300 as g
from blazingsql_gb300 import _native as N
from blazingsql_gb300.types import TypeId as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "gx_eval.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gx_[a-z_0-9]+)\s*\(", text)))


def test_header_symbols_exported():
    L = N.lib()
    syms = header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), f"{s} declared in include/gx_eval.h but not exported"
    assert sorted(N.EXPORTED_SYMBOLS) == syms


def test_version():
    assert "sm_103a" in g.version()


@pytest.mark.parametrize("cond,exprs,code", [
    ("", ["+($0, "], N.GX_ERR_PARSE),
    ("", ["FOO($0)"], N.GX_ERR_UNSUPPORTED),
    ("", ["LIKE($0, 'a%')"], N.GX_ERR_UNSUPPORTED),
    ("+($0, $1)", ["$0"], N.GX_ERR_TYPE),
    ("", ["+(1, 2)"], N.GX_ERR_UNSUPPORTED),
    ("", ["ABS(1)"], N.GX_ERR_UNSUPPORTED),
    ("", ["+($0, $7)"], N.GX_ERR_PARSE),
    ("", ["CAST(1):DOUBLE"], N.GX_ERR_TYPE),
    ("", ["+($0, 3:INTERVAL YEAR)"], N.GX_ERR_UNSUPPORTED),
])
def test_plan_errors(cond, exprs, code):
    with pytest.raises(g.GxError) as ei:
        g.Plan([T.INT64, T.FLOAT64], cond, exprs)
    assert ei.value.code == code, str(ei.value)


def test_plan_metadata():
    p = g.Plan([T.INT64, T.FLOAT64, T.INT32], "AND(>($0, 500000), <($1, 0.5), IS_NOT_NULL($2))",
               ["+(*($0, 3), $2)", "/($1, CAST($2):DOUBLE)", "$1", "7"])
    assert p.num_outputs == 4
    assert p.output_types() == [T.INT64, T.FLOAT64, T.FLOAT64, T.INT32]
    assert p.num_conjuncts == 3


PLANS = [
    # C1 plain
    ([T.INT64, T.FLOAT64, T.INT32], "AND(>($0, 500000), <($1, 0.5))", ["+(*($0, 3), $2)", "/($1, CAST($2):DOUBLE)"]),
    # every operator family at least once
    ([T.INT64, T.FLOAT64, T.TIMESTAMP_DAYS, T.INT8, T.TIMESTAMP_NANOSECONDS, T.FLOAT32], "",
     ["CASE(IS_NULL($3), FLOOR(LN(+(ABS($1), 1.0))), =($3, 0), EXP(/($1, 1000.0)), CAST($0):DOUBLE)",
      "MOD(CASE(IS_NOT_NULL($0), $0, CAST($3):BIGINT), 997)", "BL_YEAR($2)", "BL_HOUR($4)", "BL_DOW($2)",
      "OR(IS NOT TRUE(>($0, 3)), IS NOT FALSE(<($1, 0.5)))", "NOT(IS TRUE(=($3, 2)))",
      "POWER($1, 2)", "ROUND($1, 2)", "ROUND($5)", "SIN($1)", "COS($1)", "TAN($1)", "ASIN($1)", "ACOS($1)",
      "ATAN($1)", "COT($1)", "LOG10(ABS($1))", "CEIL($1)", "CAST($1):INTEGER", "CAST($0):TINYINT",
      "CAST($2):TIMESTAMP", "CAST($4):DATE", "CAST($1):FLOAT", "-($0)", "/($0, $3)", "/($1, $0)",
      "IS_NOT_DISTINCT_FROM($0, $3)", "<=($2, 1996-12-31)", ">($4, 2020-01-01 10:00:00)", "RAND()",
      "*($5, RAND())", "AND(>($0, 1), OR(<($1, 0.0), null))"]),
]


@pytest.mark.parametrize("schema,cond,exprs", PLANS)
def test_generated_kernels_compile(schema, cond, exprs):
    p = g.Plan(schema, cond or None, exprs)
    kinds = [1, 2, 3] if cond else [0]
    for masks in ([False] * len(schema), [True] * len(schema)):
        for k in kinds:
            p.compile_check(k, masks)


def test_short_circuit_kernel_compiles():
    schema = [T.INT64] * 4 + [T.FLOAT64] * 4
    cond = "AND(>($0, 10), <($4, 0.5), =($1, 3), >=($5, 1.5), <>($2, 7), <($6, 2.0))"
    p = g.Plan(schema, cond, [f"${i}" for i in range(8)], short_circuit=True, conjunct_order=[5, 4, 3, 2, 1, 0])
    p.compile_check(1, [True] * 8)
    src = p.kernel_source(1, [True] * 8)
    assert "any_alive" in src


def _gold():
    import json
    return json.load(open(os.path.join(ROOT, "tests", "golden", "reference_vectors.json")))


def test_lowering_matches_reference_strings():
    """CASE lowering / CAST renaming goldens (expression_tree_test.cpp:12-76)
    through the product's parser (and the oracle's)."""
    from oracle import pyoracle
    pairs = _gold()["case_lowering"]["pairs"]
    assert len(pairs) == 8
    for pair in pairs:
        assert N.rebuild_expression(pair["input"]) == pair["expected"]
        assert pyoracle.rebuild_expression(pair["input"]) == pair["expected"]


def test_fill_minus_op_with_zero_oracle():
    """expression_utils_test.cpp:243-278 on the oracle's restatement."""
    from oracle import pyoracle
    for pair in _gold()["fill_minus_op_with_zero"]["pairs"]:
        assert pyoracle.string_transform("fill_minus_op_with_zero", pair["input"]) == pair["expected"]
    for pair in _gold()["get_query_part"]["pairs"]:
        assert pyoracle.string_transform("get_query_part", pair["input"]) == pair["expected"]


def test_nary_and_nesting():
    """n-ary AND/OR become left-deep binary trees; OR stays n-ary next to FLOOR
    (CalciteExpressionParsing.cpp:330-398)."""
    from oracle import pyoracle
    cases = ["AND(<($0, 1), >($1, 2), =($2, 3))", "OR(=($0, 1), =($0, 2), =($0, 3), =($0, 4))",
             "AND(OR($0, $1, $2), >($1, 2), =($2, 3))", "OR(=(FLOOR($1), 1.0), =($0, 2), =($0, 3))"]
    for c in cases:
        assert N.rebuild_expression(c) == pyoracle.rebuild_expression(c), c
    assert N.rebuild_expression(cases[0]) == "AND(AND(<($0, 1), >($1, 2)), =($2, 3))"
    assert N.rebuild_expression(cases[3]).startswith("OR(=(FLOOR($1), 1.0), =($0, 2), =($0, 3))")
