"""CPU oracle of the string pre-pass and of string outputs (test infrastructure).

Restates the reference's handling of strings around its interpreter
(engine/src/execution_kernels/LogicalProject.cpp): function_evaluator_transformer
(:671-742) visits the lowered tree children first and replaces each string
operator by a synthetic column $k, computed by evaluate_string_functions
(:103-603) or evaluate_string_case_when_else (:612-659):
  - LIKE(col, 'p') (:112-133): the pattern becomes a regular expression by
    like_expression_to_regex_str (:31-47) -- '%' -> (?:.*?), '_' -> (?:.),
    '^' / '$' anchors unless the pattern starts / ends with '%' -- searched
    with cudf::strings::contains_re (here Python's re.search; '.' does not
    match a newline in either);
  - CHAR_LENGTH(col): characters per string (cudf::strings::count_characters);
  - CASE whose THEN and ELSE are string columns, string literals or null
    (FIRST_NON_MAGIC(MAGIC_IF_NOT(c, a), b), lowered as in
    parser/expression_tree.hpp:200-220, innermost pair first):
    cudf::copy_if_else(a, b, c), c evaluated by evaluate_expressions into a
    BOOL8 column; a NULL or false c selects b;
and the interpreter compares string columns with string literals or with
each other as string_view (interpreter_ops.cuh:623-719): bytes in
lexicographic order.  A NULL string gives NULL.  The rest of the expression
then runs in the C++ oracle over the table plus the synthetic columns.
An expression that is a whole string column is a string output: a copy
(LogicalProject.cpp:829, 885-887), or, under a filter, the kept rows in order
(apply_boolean_mask, LogicalFilter.cpp:22-29).  A string literal expression
is the literal repeated (:825).  Only tests/ use this module.
"""
from __future__ import annotations

import re
from typing import List, Optional, Sequence, Tuple

import numpy as np

from blazingsql_gb300.types import HostColumn, TypeId as T, pack_validity, unpack_validity
from oracle import pyoracle
from oracle.skipdata_ref import Node, parse, rebuild

CMP = {"=": "EQ", "<>": "NE", "<": "LT", "<=": "LE", ">": "GT", ">=": "GE"}
SWAP = {"<": ">", ">": "<", "<=": ">=", ">=": "<=", "=": "=", "<>": "<>"}
STRING = "string"


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


def _is_null(n: Node) -> bool:
    return not n.op and not n.var and n.value == "null"


def rewrite(texts: Sequence[str], string_cols: Sequence[int], ncols: int) -> Tuple[List[str], list]:
    """Post-order rewrite of every text; ops[i] is the column ncols + i."""
    ops: list = []
    kinds = {c: STRING for c in string_cols}

    def key(op):
        if op not in ops:
            ops.append(op)
            kinds[ncols + ops.index(op)] = STRING if op[0] == "CASE" else "num"
        return Node(f"${ncols + ops.index(op)}", var=True)

    def strcol(n):
        return n.var and kinds.get(int(n.value[1:])) == STRING

    def operand(n):
        if strcol(n):
            return ("col", int(n.value[1:]))
        if _is_null(n):
            return ("null",)
        return ("lit", _unquote(n.value))

    def walk(n: Node) -> Node:
        if not n.op:
            return n
        n.children = [walk(c) for c in n.children]
        a = n.children
        if n.value == "LIKE" and len(a) == 2 and strcol(a[0]) and _is_lit(a[1]):
            return key(("LIKE", int(a[0].value[1:]), _unquote(a[1].value)))
        if n.value == "CHAR_LENGTH" and len(a) == 1 and strcol(a[0]):
            return key(("CHAR_LENGTH", int(a[0].value[1:]), ""))
        if n.value in CMP and len(a) == 2 and (strcol(a[0]) or strcol(a[1])) and \
                all(strcol(x) or _is_lit(x) for x in a):
            sw = not strcol(a[0])
            op = SWAP[n.value] if sw else n.value
            c, r = (a[1], a[0]) if sw else (a[0], a[1])
            rhs = ("col", int(r.value[1:])) if strcol(r) else _unquote(r.value)
            return key((CMP[op], int(c.value[1:]), rhs))
        if n.value == "CASE" and len(a) >= 3 and len(a) % 2 == 1:
            cur = a[-1]
            i = len(a) - 1
            folded = False

            def stringish(x):
                return strcol(x) or _is_lit(x) or _is_null(x)
            while i >= 2 and stringish(a[i - 1]) and stringish(cur) and not (_is_null(a[i - 1]) and _is_null(cur)):
                cond = a[i - 2]
                if not cond.op and not cond.var:
                    raise ValueError("CASE operator not supported for condition expression literals")
                cur = key(("CASE", rebuild(cond, typed=True), operand(a[i - 1]), operand(cur)))
                folded = True
                i -= 2
            if not folded:
                return n
            if i == 0:
                return cur
            n.children = a[:i] + [cur]
            return n
        return n

    def check(n: Node, top: bool):
        if (strcol(n) or _is_lit(n)) and not top:
            raise ValueError("string column or literal outside a string operator")
        for c in n.children if n.op else []:
            check(c, False)

    out = []
    for t in texts:
        if not t:
            out.append(t)
            continue
        root = walk(parse(t))
        check(root, True)
        out.append(rebuild(root, typed=True))
    return out, ops


def evaluate_op(op, values: Sequence[Optional[str]], values2: Optional[Sequence[Optional[str]]] = None
                ) -> HostColumn:
    """One non-CASE operator over a string column (values2: the right-hand
    column of a comparison of two columns)."""
    kind, _, lit = op
    valid = np.array([v is not None for v in values])
    if kind == "CHAR_LENGTH":
        data = np.array([len(v) if v is not None else 0 for v in values], dtype=np.int32)
        return HostColumn(T.INT32, data, pack_validity(valid))
    if kind == "LIKE":
        rx = re.compile(_py_regex(like_to_regex(lit)))
        data = [v is not None and rx.search(v) is not None for v in values]
    else:
        f = {"EQ": lambda x, y: x == y, "NE": lambda x, y: x != y, "LT": lambda x, y: x < y,
             "LE": lambda x, y: x <= y, "GT": lambda x, y: x > y, "GE": lambda x, y: x >= y}[kind]
        if values2 is None:
            b = lit.encode("utf-8")
            data = [v is not None and f(v.encode("utf-8"), b) for v in values]
        else:
            valid = valid & np.array([v is not None for v in values2])
            data = [ok and f(v.encode("utf-8"), w.encode("utf-8")) for ok, v, w in zip(valid, values, values2)]
    return HostColumn(T.BOOL8, np.array(data, dtype=np.uint8), pack_validity(valid))


def _numeric_table(cols, strings: dict, n: int):
    """The table as the C++ oracle sees it: string columns become INT8
    placeholders (nothing reads them after the rewrite)."""
    return [HostColumn(T.INT8, np.zeros(n, dtype=np.int8)) if i in strings else c for i, c in enumerate(cols)]


def _truthy(col: HostColumn) -> np.ndarray:
    n = len(col.data)
    valid = unpack_validity(col.mask, n) if col.mask is not None else np.ones(n, dtype=bool)
    return valid & (np.asarray(col.data) != 0)


def prepass(cols: Sequence, strings: dict, texts: Sequence[str], nthreads: int = 4):
    """(rewritten texts, table with synthetic columns, string columns by position)."""
    n = len(next(iter(strings.values()))) if strings else len(cols[0].data)
    texts, ops = rewrite(list(texts), list(strings), len(cols))
    strings = dict(strings)
    table = _numeric_table(cols, strings, n)
    for op in ops:
        k = len(table)
        if op[0] == "CASE":
            cond = pyoracle.evaluate_expressions(table, [op[1]], nthreads)[0]
            if cond.type_id != T.BOOL8:
                raise ValueError("Expression does not evaluate to a boolean mask")
            pick = _truthy(cond)

            def src(o):
                if o[0] == "col":
                    return strings[o[1]]
                return [None if o[0] == "null" else o[1]] * n
            a, b = src(op[2]), src(op[3])
            strings[k] = [a[i] if pick[i] else b[i] for i in range(n)]
            table.append(HostColumn(T.INT8, np.zeros(n, dtype=np.int8)))
        else:
            rhs = op[2]
            if isinstance(rhs, tuple):
                table.append(evaluate_op((op[0], op[1], ""), strings[op[1]], strings[rhs[1]]))
            else:
                table.append(evaluate_op(op, strings[op[1]]))
    return texts, table, strings


def _string_output(text: str, strings: dict):
    """The strings of a string output expression, or None for a plan output."""
    t = text.strip()
    if re.fullmatch(r"\$\d+", t) and int(t[1:]) in strings:
        return strings[int(t[1:])]
    if t.startswith("'"):
        return _unquote(t[:t.rindex("'") + 1])
    return None


def evaluate_expressions(cols: Sequence, strings: dict, exprs: Sequence[str], nthreads: int = 4):
    """cols: HostColumns (None at string positions); strings: position -> list
    of str / None.  Returns HostColumns, or lists of strings for string outputs."""
    n = len(next(iter(strings.values()))) if strings else len(cols[0].data)
    texts, table, strings = prepass(cols, strings, exprs, nthreads)
    outs: list = [None] * len(texts)
    num = []
    for i, t in enumerate(texts):
        s = _string_output(t, strings)
        if s is None:
            num.append(i)
        else:
            outs[i] = list(s) if isinstance(s, list) else [s] * n
    if num:
        for i, c in zip(num, pyoracle.evaluate_expressions(table, [texts[i] for i in num], nthreads)):
            outs[i] = c
    return outs


def filter_project(cols: Sequence, strings: dict, condition: str, exprs: Sequence[str], nthreads: int = 4):
    """(outputs, surviving rows); string outputs are lists of str / None."""
    texts, table, strings = prepass(cols, strings, [condition] + list(exprs), nthreads)
    cond, texts = texts[0], texts[1:]
    keep = np.flatnonzero(_truthy(pyoracle.evaluate_expressions(table, [cond], nthreads)[0]))
    outs: list = [None] * len(texts)
    num = []
    for i, t in enumerate(texts):
        s = _string_output(t, strings)
        if s is None:
            num.append(i)
        else:
            outs[i] = [s[r] for r in keep] if isinstance(s, list) else [s] * len(keep)
    if num:
        got, rows = pyoracle.filter_project(table, cond, [texts[i] for i in num], nthreads)
        assert rows == len(keep)
        for i, c in zip(num, got):
            outs[i] = c
    return outs, len(keep)


def process_filter(cols: Sequence, strings: dict, condition: str, nthreads: int = 4):
    """Every column compacted by the condition (LogicalFilter.cpp:31-52)."""
    return filter_project(cols, strings, condition, [f"${i}" for i in range(len(cols))], nthreads)
