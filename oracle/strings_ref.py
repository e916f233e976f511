"""CPU oracle of the string pre-pass (test infrastructure).

Restates the reference's handling of string operators before its
interpreter runs (engine/src/execution_kernels/LogicalProject.cpp):
function_evaluator_transformer (:671-742) replaces each string operator by a
synthetic column $k, computed by evaluate_string_functions (:103-603):
  - LIKE(col, 'p') (:112-133): the pattern becomes a regular expression by
    like_expression_to_regex_str (:31-47) -- '%' -> (?:.*?), '_' -> (?:.),
    '^' / '$' anchors unless the pattern starts / ends with '%' -- searched
    with cudf::strings::contains_re (here Python's re.search; '.' does not
    match a newline in either);
  - CHAR_LENGTH(col): characters per string (cudf::strings::count_characters);
and the interpreter compares a string column with a string literal as
string_view (interpreter_ops.cuh:623-719): bytes in lexicographic order.
A NULL string gives NULL.  The rest of the expression then runs in the C++
oracle over the table plus the synthetic columns.  Only tests/ use this module.
"""
from __future__ import annotations

import re
from typing import List, Optional, Sequence, Tuple

import numpy as np

from blazingsql_gb300.types import HostColumn, TypeId as T, pack_validity
from oracle import pyoracle
from oracle.skipdata_ref import Node, parse, rebuild

CMP = {"=": "EQ", "<>": "NE", "<": "LT", "<=": "LE", ">": "GT", ">=": "GE"}
SWAP = {"<": ">", ">": "<", "<=": ">=", ">=": "<=", "=": "=", "<>": "<>"}


def like_to_regex(p: str) -> str:
    """like_expression_to_regex_str (LogicalProject.cpp:31-47) for patterns
    without regular-expression characters."""
    if not p:
        return p
    start, end = p[0] != "%", p[-1] != "%"
    r = p.replace("%", "(?:.*?)").replace("_", "(?:.)")
    return ("^" if start else "") + r + ("$" if end else "")


def _py_regex(rx: str) -> str:
    # '$' at the very end of the string (Python's '$' also matches before a final newline)
    return rx[:-1] + r"\Z" if rx.endswith("$") else rx


def _unquote(t: str) -> str:
    return t[1:-1].replace("''", "'") if len(t) >= 2 and t[0] in "'\"" and t[-1] == t[0] else t


def _is_lit(n: Node) -> bool:
    return not n.op and not n.var and n.value[:1] in ("'", '"')


def rewrite(texts: Sequence[str], string_cols: Sequence[int], ncols: int) -> Tuple[List[str], list]:
    ops: list = []

    def key(op):
        if op not in ops:
            ops.append(op)
        return f"${ncols + ops.index(op)}"

    def strcol(n):
        return n.var and int(n.value[1:]) in string_cols

    def walk(n: Node) -> Node:
        if n.var:
            if strcol(n):
                raise ValueError("string column outside the pre-pass")
            return n
        if not n.op:
            return n
        a = n.children
        if n.value == "LIKE" and len(a) == 2 and strcol(a[0]) and _is_lit(a[1]):
            return Node(key(("LIKE", int(a[0].value[1:]), _unquote(a[1].value))), var=True)
        if n.value == "CHAR_LENGTH" and len(a) == 1 and strcol(a[0]):
            return Node(key(("CHAR_LENGTH", int(a[0].value[1:]), "")), var=True)
        if n.value in CMP and len(a) == 2 and ((strcol(a[0]) and _is_lit(a[1])) or (_is_lit(a[0]) and strcol(a[1]))):
            sw = not strcol(a[0])
            op = SWAP[n.value] if sw else n.value
            c, lit = (a[1], a[0]) if sw else (a[0], a[1])
            return Node(key((CMP[op], int(c.value[1:]), _unquote(lit.value))), var=True)
        n.children = [walk(c) for c in a]
        return n

    out = []
    for t in texts:
        if not t:
            out.append(t)
            continue
        out.append(rebuild(walk(parse(t))))
    return out, ops


def evaluate_op(op, values: Sequence[Optional[str]]) -> HostColumn:
    kind, _, lit = op
    valid = np.array([v is not None for v in values])
    if kind == "CHAR_LENGTH":
        data = np.array([len(v) if v is not None else 0 for v in values], dtype=np.int32)
        return HostColumn(T.INT32, data, pack_validity(valid))
    if kind == "LIKE":
        rx = re.compile(_py_regex(like_to_regex(lit)))
        data = [v is not None and rx.search(v) is not None for v in values]
    else:
        b = lit.encode("utf-8")
        f = {"EQ": lambda x: x == b, "NE": lambda x: x != b, "LT": lambda x: x < b, "LE": lambda x: x <= b,
             "GT": lambda x: x > b, "GE": lambda x: x >= b}[kind]
        data = [v is not None and f(v.encode("utf-8")) for v in values]
    return HostColumn(T.BOOL8, np.array(data, dtype=np.uint8), pack_validity(valid))


def _table(cols, strings):
    """The numeric table plus the synthetic columns: string columns become
    INT8 placeholders (nothing reads them after the rewrite)."""
    n = len(next(iter(strings.values()))) if strings else len(cols[0].data)
    return [HostColumn(T.INT8, np.zeros(n, dtype=np.int8)) if i in strings else c for i, c in enumerate(cols)]


def filter_project(cols: Sequence, strings: dict, condition: str, exprs: Sequence[str], nthreads: int = 4):
    """cols: HostColumns (None at string positions); strings: position -> list of str / None."""
    texts, ops = rewrite([condition] + list(exprs), list(strings), len(cols))
    table = _table(cols, strings) + [evaluate_op(op, strings[op[1]]) for op in ops]
    out, rows = pyoracle.filter_project(table, texts[0], texts[1:], nthreads)
    return out, rows


def evaluate_expressions(cols: Sequence, strings: dict, exprs: Sequence[str], nthreads: int = 4):
    texts, ops = rewrite(list(exprs), list(strings), len(cols))
    table = _table(cols, strings) + [evaluate_op(op, strings[op[1]]) for op in ops]
    return pyoracle.evaluate_expressions(table, texts, nthreads)
