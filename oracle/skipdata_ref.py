"""CPU oracle of the skip-data (row-group pruning) predicate (test infrastructure).

Restates ral::skip_data (engine/src/skip_data/SkipDataProcessor.cpp):
  - drop_value (:215-218, transformer :23-45): operands of columns without
    statistics become NONE;
  - apply_skip_data_rules (:220-232): the reducer (:167-212, with
    is_unsupported_binary_op / is_exclusion_unary_op of skip_data/utils.cpp:12-37)
    removes operators other than = > >= < <= + - AND OR (an AND keeps the other
    side of a removed operand, any other operator is removed with it); an
    unusable root (NONE) ends the rewrite; then the transformer (:48-165)
    restates each comparison over $2i (min) and $2i+1 (max): = -> AND(<=(n.min,
    m.max), >=(n.max, m.min)); < <= -> op(n.min, m.max); > >= -> op(n.max,
    m.min); + - -> "&&&"(op(n.min, m.min), op(n.max, m.max)), whose min / max
    halves comparisons above pick;
  - process_skipdata_for_table (:252-350): the rewritten condition evaluated
    over the metadata table's [min, max] pairs keeps the (file, row group) ids
    of the rows where it is true.
Checked against the reference's own tests (engine/tests/skipdata/
expression_tree_test.cpp, extracted into tests/golden/reference_vectors.json).
The parse handles the RexNode subset those conditions use: NAME(args...),
$n and literals; n-ary AND / OR nest left-deep first
(CalciteExpressionParsing.cpp:330-398).  Only tests/ use this module.
"""
from __future__ import annotations

import re
from typing import List, Optional, Sequence, Tuple

SUPPORTED = {"=", ">", ">=", "<", "<=", "+", "-", "AND", "OR"}


class Node:
    def __init__(self, value: str, children: Optional[list] = None, var: bool = False):
        self.value = value
        self.children = children or []
        self.var = var
        self.op = not var and children is not None

    def __repr__(self):
        return prefix(self)


def _none() -> Node:
    return Node("NONE", [])


def parse(text: str, fn_types: bool = False) -> Node:
    """fn_types: a function's result type ("CAST($0):VARCHAR") joins its name
    ("CAST_VARCHAR"), as the evaluator's parser names such operators."""
    s = text.strip()
    pos = 0

    def skip():
        nonlocal pos
        while pos < len(s) and s[pos] == " ":
            pos += 1

    def expr() -> Node:
        nonlocal pos
        skip()
        if s[pos] == "$":
            m = re.match(r"\$\d+", s[pos:])
            pos += m.end()
            return Node(m.group(0), var=True)
        m = re.match(r"[A-Za-z_][A-Za-z_ ]*(?=\()|[=<>+\-*/|]+(?=\()", s[pos:])
        if m:
            name = m.group(0).strip()
            pos += m.end() + 1
            args = []
            skip()
            if s[pos] != ")":
                args.append(expr())
                skip()
                while s[pos] == ",":
                    pos += 1
                    args.append(expr())
                    skip()
            pos += 1
            if fn_types and pos < len(s) and s[pos] == ":":
                m = re.match(r":([A-Z_]+)", s[pos:])
                pos += m.end()
                name += "_" + m.group(1)
            return Node(name, args)
        m = re.match(r"'[^']*'(?::[A-Z]+)?|[^,()\s]+", s[pos:])
        pos += m.end()
        tok = m.group(0)
        if tok.startswith("'"):
            q = tok.rindex("'")
            n = Node(tok[:q + 1])
            n.suffix = tok[q + 2:]
        else:
            n = Node(tok.split(":")[0])
            n.suffix = tok.split(":", 1)[1] if ":" in tok else ""
        return n

    root = expr()
    return _nest(root)


def _nest(n: Node) -> Node:
    if n.op:
        n.children = [_nest(c) for c in n.children]
        if n.value in ("AND", "OR") and len(n.children) > 2:
            acc = Node(n.value, n.children[:2])
            for c in n.children[2:]:
                acc = Node(n.value, [acc, c])
            return acc
    return n


def drop(n: Node, v: str) -> Node:
    if n.op:
        n.children = [drop(c, v) for c in n.children]
    return _none() if n.value == v else n


def _exclusion(n: Node) -> bool:
    # children are reduced first: a removed operand or unary operator is NONE by now
    return n.op and (n.value == "NONE" or (n.value not in SUPPORTED and len(n.children) <= 1))


def reduce(n: Node) -> Node:
    if not n.op:
        return n
    n.children = [reduce(c) for c in n.children]
    if n.value not in SUPPORTED or len(n.children) != 2:
        return _none()
    a, b = n.children
    la, lb = _exclusion(a), _exclusion(b)
    if la and not lb:
        return b if n.value == "AND" else _none()
    if lb and not la:
        return a if n.value == "AND" else _none()
    if la and lb:
        return _none()
    return n


def _inc(n: Node, k: int) -> Node:
    if n.var:
        return Node("$" + str(2 * int(n.value[1:]) + k), var=True)
    if n.op and n.value == "&&&":
        return n.children[k]
    return n


def transform(n: Node) -> Node:
    if not n.op:
        return n
    n.children = [transform(c) for c in n.children]
    if len(n.children) != 2:
        return n
    a, b = n.children
    v = n.value
    if v == "=":
        return Node("AND", [Node("<=", [_inc(a, 0), _inc(b, 1)]), Node(">=", [_inc(a, 1), _inc(b, 0)])])
    if v in ("<", "<="):
        return Node(v, [_inc(a, 0), _inc(b, 1)])
    if v in (">", ">="):
        return Node(v, [_inc(a, 1), _inc(b, 0)])
    if v in ("+", "-"):
        return Node("&&&", [Node(v, [_inc(a, 0), _inc(b, 0)]), Node(v, [_inc(a, 1), _inc(b, 1)])])
    return n


def prefix(n: Node) -> str:
    if n.op and n.value:
        ops = " ".join(prefix(c) for c in n.children)
        return n.value + (" " + ops if ops else "")
    return n.value


def rebuild(n: Node, typed: bool = False) -> str:
    """Text of a tree; typed keeps literals' explicit ":TYPE"."""
    if n.op:
        return n.value + "(" + ", ".join(rebuild(c, typed) for c in n.children) + ")"
    suffix = getattr(n, "suffix", "")
    return n.value + (":" + suffix if typed and suffix and not n.var else "")


def rewrite(condition: str, dropped: Sequence[int] = ()) -> Tuple[str, str]:
    """(rewritten condition text or "" when unusable, prefix form)."""
    t = parse(condition)
    for c in dropped:
        t = drop(t, f"${c}")
    t = reduce(t)
    if t.value == "NONE":
        return "", "NONE"
    t = transform(t)
    return rebuild(t), prefix(t)


def row_groups(metadata: dict, names: List[str], table_scan_condition: str, projected: Sequence[int],
               ids: Tuple[Sequence[int], Sequence[int]]):
    """(file, row group) ids kept by the rewritten condition, or None when it
    allows no pruning.  metadata: name -> numpy column; the evaluation goes
    through the C++ oracle."""
    import numpy as np
    from blazingsql_gb300.types import HostColumn, TypeId as T, unpack_validity
    from oracle import pyoracle
    cols, dropped = [], []
    nrows = len(ids[0])
    for i, c in enumerate(projected):
        mn, mx = f"min_{c}_{names[c]}", f"max_{c}_{names[c]}"
        if mn in metadata and mx in metadata:
            cols += [metadata[mn], metadata[mx]]
        else:
            dropped.append(i)
            cols += [HostColumn(T.INT8, np.zeros(nrows, dtype=np.int8))] * 2
    text, _ = rewrite(table_scan_condition, dropped)
    if not text:
        return None
    k = len(cols)
    cols += [HostColumn(T.INT32, np.asarray(ids[0], dtype=np.int32)), HostColumn(T.INT32, np.asarray(ids[1], dtype=np.int32))]
    out, rows = pyoracle.filter_project(cols, text, [f"${k}", f"${k + 1}"])
    return list(out[0].data[:rows]), list(out[1].data[:rows])
