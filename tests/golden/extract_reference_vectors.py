"""Extract BlazingSQL's own known-answer vectors for the row-wise evaluator.

Reads the reference's gtest sources as text (they cannot run here: they need
libcudf) and writes ``reference_vectors.json`` beside this script.  Every entry
records the file and line range it came from.  Run from the repo root:

    python tests/golden/extract_reference_vectors.py /path/to/blazingsql

The committed JSON is what the tests use; this script only regenerates it.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _lines(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read().split("\n")


def _numbers(text):
    return [float(x) if ("." in x or "e" in x) else int(x) for x in re.findall(r"-?\d+(?:\.\d+)?(?:e-?\d+)?", text)]


def _wrapper_list(lines, a, b, var):
    """Values of `var`'s first brace list (wrapper declared between lines a..b, 1-based)."""
    text = "\n".join(lines[a - 1:b])
    m = re.search(re.escape(var) + r"\s*[\({]\s*\{([^}]*)\}", text)
    if not m:
        raise ValueError(f"{var} not found in lines {a}-{b}")
    return _numbers(m.group(1))


def _wrapper_valid(lines, a, b, var):
    text = "\n".join(lines[a - 1:b])
    m = re.search(re.escape(var) + r"\s*[\({]\s*\{[^}]*\}\s*,\s*\{([^}]*)\}", text)
    return _numbers(m.group(1)) if m else None


def _string_pairs(lines, a, b, build_pat, exp_pat):
    text = "\n".join(lines[a - 1:b])
    builds = re.findall(build_pat, text)
    exps = re.findall(exp_pat, text)
    return [{"input": x, "expected": y} for x, y in zip(builds, exps)]


def extract(root):
    out = {}
    it = "engine/tests/new-tests/interops_tests.cpp"
    L = _lines(root, it)
    out["interops_numeric"] = {
        "source": f"{it}:199-278",
        "expected_col1": _wrapper_list(L, 271, 272, "expected_col1"),
        "expected_col2": _wrapper_list(L, 273, 274, "expected_col2"),
    }
    out["interops_day_of_week"] = {
        "source": f"{it}:294-363",
        "start_ms": -2203891200000, "stop_ms": 2214086400000, "rows": 20,
        "expected_days": _wrapper_list(L, 351, 352, "expected_col1"),
        "expected_other": _wrapper_list(L, 357, 358, "expected_col1"),
    }
    comp = {"source": f"{it}:457-557", "start_ms": -2500000000000, "stop_ms": 2500000000000, "rows": 10,
            "days": {}, "other": {}}
    for k in range(1, 8):
        comp["days"][f"col{k}"] = _wrapper_list(L, 529, 536, f"expected_col{k}")
        comp["other"][f"col{k}"] = _wrapper_list(L, 543, 550, f"expected_col{k}")
    out["interops_timestamp_components"] = comp

    pp = "engine/tests/new-tests/process_project.cpp"
    L = _lines(root, pp)
    out["project_inputs"] = {"source": f"{pp}:16-200",
                             "col1": _wrapper_list(L, 20, 20, "col1"), "col3": _wrapper_list(L, 22, 22, "col3")}
    out["project_gt3"] = {"source": f"{pp}:129-160",
                          "bool": _wrapper_list(L, 152, 152, "expect_col1"),
                          "other": _wrapper_list(L, 157, 157, "expect_col1")}
    out["project_gt3_lt3"] = {"source": f"{pp}:162-199",
                              "bool_col1": _wrapper_list(L, 187, 187, "expect_col1"),
                              "bool_col3": _wrapper_list(L, 188, 188, "expect_col3"),
                              "other_col1": _wrapper_list(L, 193, 193, "expect_col1"),
                              "other_col3": _wrapper_list(L, 194, 194, "expect_col3")}
    out["project_round"] = {"source": f"{pp}:492-513",
                            "input": _wrapper_list(L, 496, 496, "col1"),
                            "round0": _wrapper_list(L, 507, 507, "expect_col1"),
                            "round2": _wrapper_list(L, 508, 508, "expect_col2"),
                            "round5": _wrapper_list(L, 509, 509, "expect_col3")}

    af = "engine/tests/new-tests/apply_filter.cpp"
    L = _lines(root, af)
    out["apply_filter_with_null"] = {
        "source": f"{af}:44-86",
        "col1": _wrapper_list(L, 51, 51, "col1"), "col1_valid": _wrapper_valid(L, 51, 51, "col1"),
        "col3": _wrapper_list(L, 53, 53, "col3"), "col3_valid": _wrapper_valid(L, 53, 53, "col3"),
        "mask": _wrapper_list(L, 61, 61, "bool_filter"), "mask_valid": _wrapper_valid(L, 61, 61, "bool_filter"),
        "expect_col1": _wrapper_list(L, 69, 69, "expect_col1"),
        "expect_col1_valid": _wrapper_valid(L, 69, 69, "expect_col1"),
        "expect_col3": _wrapper_list(L, 71, 71, "expect_col3"),
        "expect_col3_valid": _wrapper_valid(L, 71, 71, "expect_col3"),
    }

    et = "engine/tests/parser/expression_tree_test.cpp"
    L = _lines(root, et)
    out["case_lowering"] = {
        "source": f"{et}:12-76",
        "pairs": _string_pairs(L, 12, 76, r'tree\.build\("([^"]*)"\)', r'(?:std::string expected =\s*)"([^"]*)"'),
    }
    eu = "engine/tests/parser/expression_utils_test.cpp"
    L = _lines(root, eu)
    pairs = []
    text = "\n".join(L[242:278])
    for blk in re.split(r"TEST_F", text)[1:]:
        e = re.search(r'std::string expression = "([^"]*)"', blk)
        x = re.search(r'std::string expected_expression = "([^"]*)"', blk)
        if e:
            pairs.append({"input": e.group(1), "expected": x.group(1) if x else e.group(1)})
    out["fill_minus_op_with_zero"] = {"source": f"{eu}:243-278", "pairs": pairs}
    # preprocess rewrites: convert_ms_to_ns_units and reinterpret_timestamp,
    # each test's input, expected text (its input when it expects no change)
    # and schema (cudf type names, in order)
    text = "\n".join(L)
    pre = []
    for m in re.finditer(r"TEST_F\(ExpressionUtilsTest, (\w+)\)", text):
        nxt = text.find("TEST_F(", m.end())
        blk = text[m.start():nxt if nxt >= 0 else len(text)]
        fn = re.search(r"out_expression = (convert_ms_to_ns_units|reinterpret_timestamp)\(", blk)
        if not fn:
            continue
        inp = re.search(r'std::string expression = "(.*)";', blk).group(1)
        exp = re.search(r'std::string expected_str = "(.*)";', blk)
        first = text.count("\n", 0, m.start()) + 1
        pre.append({"name": m.group(1), "function": fn.group(1), "input": inp,
                    "expected": exp.group(1) if exp else inp,
                    "schema": re.findall(r"cudf::type_id::(\w+)", blk),
                    "source": f"{eu}:{first}-{first + blk.count(chr(10))}"})
    out["preprocess_rewrites"] = pre
    gq = [i for i, l in enumerate(L) if "getting_query_part" in l][0]
    blk = "\n".join(L[gq:gq + 14])
    out["get_query_part"] = {"source": f"{eu}:{gq + 1}-{gq + 14}",
                             "pairs": [{"input": re.search(r'query_part_%d = "(.*)";' % k, blk).group(1),
                                        "expected": re.search(r'expected_%d = "(.*)";' % k, blk).group(1)}
                                       for k in (1, 2)]}
    # skip-data rewrite: the prefix-notation trees of the reference's tests,
    # with the operands dropped before the rules where a test drops some
    sd = "engine/tests/skipdata/expression_tree_test.cpp"
    L = _lines(root, sd)
    text = "\n".join(L)
    cases = []
    for m in re.finditer(r"TEST_F\(ExpressionTreeTest, (\w+)\)", text):
        start = m.start()
        nxt = text.find("TEST_F(", m.end())
        blk = text[start:nxt if nxt >= 0 else len(text)]
        # tests commented out line by line start with //
        line_start = text.rfind("\n", 0, start) + 1
        if text[line_start:start].strip().startswith("//"):
            continue
        pre = re.search(r'std::string prefix = "([^"]*)"', blk)
        exp = re.search(r'std::string expected = "([^"]*)"', blk)
        if not pre or not exp:
            continue
        drops = [int(x) for x in re.findall(r'drop_value\(tree, "\$(\d+)"\)', blk)]
        first = text.count("\n", 0, start) + 1
        last = first + blk.count("\n")
        cases.append({"name": m.group(1), "input": pre.group(1), "expected": exp.group(1), "dropped": drops,
                      "source": f"{sd}:{first}-{last}"})
    out["skip_data_rewrite"] = {"source": sd, "cases": cases}
    # tables with string columns: filters that compact them and CASEs with
    # string results (their inputs, query and expected columns)
    out["string_tables"] = [
        _string_table_test(root, "engine/tests/new-tests/filter_tests.cpp", "LogicalFilterWithStringsTest", "NoNulls"),
        _string_table_test(root, "engine/tests/new-tests/filter_tests.cpp", "LogicalFilterWithStringsTest",
                           "IneqWithNulls"),
        _string_table_test(root, "engine/tests/new-tests/process_project.cpp", "ProjectTestString",
                           "test_string_case"),
        _string_table_test(root, "engine/tests/new-tests/process_project.cpp", "ProjectTestString",
                           "test_string_nested_case"),
    ] + [_string_table_test(root, "engine/tests/new-tests/process_project.cpp", "ProjectTestString", t)
         for t in ("test_string_like", "test_string_substring", "test_string_substring_null", "test_char_length",
                   "test_string_concat", "test_cast_to_string", "test_cast_from_string")]
    return out


def _brace_groups(text):
    """Top-level {...} groups of a wrapper's argument text."""
    groups, depth, start = [], 0, None
    for i, ch in enumerate(text):
        if ch == '"':
            continue
        if ch == "{":
            depth += 1
            if depth == 1 or (depth == 2 and text.lstrip().startswith("{{")):
                start = i + 1
        elif ch == "}":
            if start is not None and (depth == 1 or (depth == 2 and text.lstrip().startswith("{{"))):
                groups.append(text[start:i])
                start = None
            depth -= 1
    return groups


def _wrapper_columns(block):
    cols = []
    pat = r'(strings_column_wrapper|fixed_width_column_wrapper<([^>]*)>)\s+(\w+)\s*[\({](.*?)[\)}];'
    for m in re.finditer(pat, block, re.S):
        # element type: bool, int32_t, double, ...; timestamp wrappers
        # (cudf::timestamp_s, cudf::timestamp_s::rep) by their unit
        kind = "string" if m.group(1).startswith("strings") else m.group(2).split(",")[0].strip().replace("cudf::", "")
        body = m.group(4)
        groups = _brace_groups(body)
        if kind == "string":
            values = [bytes(v, "utf-8").decode("unicode_escape") for v in re.findall(r'"((?:[^"\\]|\\.)*)"', groups[0])]
        elif kind == "bool":
            words = re.findall(r"true|false", groups[0])
            values = [1 if w == "true" else 0 for w in words] if words else _numbers(groups[0])
        else:
            values = _numbers(groups[0])
        valid = _numbers(groups[1]) if len(groups) > 1 else None
        cols.append({"name": m.group(3), "kind": kind, "values": values, "valid": valid})
    return cols


def _string_table_test(root, rel, fixture, name):
    L = _lines(root, rel)
    text = "\n".join(L)
    m = re.search(r"TEST_F\(%s, %s\)" % (fixture, name), text)
    nxt = text.find("TEST_F(", m.end())
    end = nxt if nxt >= 0 else len(text)
    nxt_t = text.find("template", m.end())
    if 0 <= nxt_t < end:
        end = nxt_t
    blk = text[m.start():end]
    first = text.count("\n", 0, m.start()) + 1
    last = first + blk.rstrip().count("\n")
    cols = _wrapper_columns(blk)
    query = re.search(r'"(Logical\w+\(.*?\))"', blk).group(1)
    return {"name": f"{fixture}.{name}", "source": f"{rel}:{first}-{last}", "query": query,
            "inputs": [c for c in cols if not c["name"].startswith("expected")],
            "expected": [c for c in cols if c["name"].startswith("expected")]}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BLAZINGSQL_SRC", "")
    if not root or not os.path.isdir(root):
        sys.exit("usage: extract_reference_vectors.py <blazingsql source root>")
    data = extract(root)
    with open(os.path.join(HERE, "reference_vectors.json"), "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", os.path.join(HERE, "reference_vectors.json"))


if __name__ == "__main__":
    main()
