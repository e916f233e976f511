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
  - SUBSTRING / LEFT / RIGHT / REVERSE: cudf::strings::slice_strings by
    characters with the start / stop of :186-220 and :573-585;
  - CONCAT / || (n-ary CONCAT nested to the left first,
    expression_utils.cpp:1620): NULL if either side is;
  - TRIM (strip of the given characters, or of characters <= ' ' when none
    are given), REPLACE (every occurrence, left to right), UPPER / LOWER /
    INITCAP (ASCII);
  - CAST to VARCHAR (cast_to_str_functor, :62-92): "true" / "false", decimal
    integers, "%Y-%m-%d" for dates and "%Y-%m-%d %H:%M:%S" for timestamps;
  - CAST of a string column to an integer (cudf::strings::to_integers: an
    optional sign, then digits up to the first other character, wrapped to
    the type) or to DATE / TIMESTAMP (to_timestamps with "%Y-%m-%d" /
    "%Y-%m-%d %H:%M:%S": each field read from its place in the format, up to
    its first non-digit, 0 past the end of the string);
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

import math
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
            kinds[ncols + ops.index(op)] = STRING if op[0] in STRING_RESULTS else "num"
        return Node(f"${ncols + ops.index(op)}", var=True)

    def strcol(n):
        return n.var and kinds.get(int(n.value[1:])) == STRING

    def operand(n):
        if strcol(n):
            return ("col", int(n.value[1:]))
        if _is_null(n):
            return ("null",)
        return ("lit", _unquote(n.value))

    def int_lit(x):
        if x.op or x.var or not re.fullmatch(r"-?\d+", x.value):
            raise ValueError("non-literal position")
        return int(x.value)

    def walk(n: Node) -> Node:
        if not n.op:
            return n
        if n.value == "CONCAT" and len(n.children) > 2:
            cur = n.children[0]
            for c in n.children[1:]:
                cur = Node("CONCAT", [cur, c])
            n = cur
        n.children = [walk(c) for c in n.children]
        a = n.children
        fn = string_function(n.value, a, strcol, int_lit)
        if fn is not None:
            return key(fn)
        if n.value in ("CAST_VARCHAR", "CAST_CHAR") and len(a) == 1 and not a[0].op and not a[0].var \
                and not _is_null(a[0]):
            return Node(a[0].value if _is_lit(a[0]) else "'" + a[0].value + "'")
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
        for side in ("BOTH", "LEADING", "TRAILING"):  # replace_calcite_regex (expression_utils.cpp:1096-1098)
            t = t.replace(f"TRIM(FLAG({side}),", f'TRIM("{side}",')
        root = walk(parse(t, fn_types=True))
        check(root, True)
        out.append(rebuild(root, typed=True))
    return out, ops


STRING_RESULTS = {"CASE", "SLICE", "SLICE_COLS", "UPPER", "LOWER", "INITCAP", "TRIM", "REPLACE", "CONCAT",
                  "TO_STRING", "REGEX"}
PARSE_TYPES = {"CAST_TINYINT": T.INT8, "CAST_SMALLINT": T.INT16, "CAST_INTEGER": T.INT32, "CAST_BIGINT": T.INT64,
               "CAST_DATE": T.TIMESTAMP_DAYS, "CAST_TIMESTAMP_SECONDS": T.TIMESTAMP_SECONDS,
               "CAST_TIMESTAMP_MILLISECONDS": T.TIMESTAMP_MILLISECONDS,
               "CAST_TIMESTAMP_MICROSECONDS": T.TIMESTAMP_MICROSECONDS, "CAST_TIMESTAMP": T.TIMESTAMP_NANOSECONDS,
               "CAST_FLOAT": T.FLOAT32, "CAST_DOUBLE": T.FLOAT64}


def string_function(name, a, strcol, int_lit):
    """The operator tuple of one of evaluate_string_functions' functions, or None."""
    if name == "SUBSTRING" and len(a) in (2, 3) and strcol(a[0]):
        def lit(x):
            try:
                return int_lit(x)
            except ValueError:
                return None
        if lit(a[1]) is not None and (len(a) == 2 or lit(a[2]) is not None):
            start = max(int_lit(a[1]), 1) - 1
            length = int_lit(a[2]) if len(a) == 3 else -1
            return ("SLICE", int(a[0].value[1:]), start, start + length if length >= 0 else None, 1)
        # positions from columns or expressions (LogicalProject.cpp:221-300): a
        # literal start is max(start, 1), any start then 1 less (zero-based,
        # transform_start_to_zero_based_indexing), the stop start + length
        # (transform_length_to_end), no length: to the end
        st = lit(a[1])
        start = str(max(st, 1) - 1) if st is not None else "-(" + rebuild(a[1], typed=True) + ", 1)"
        stop = "+(" + start + ", " + rebuild(a[2], typed=True) + ")" if len(a) == 3 else None
        return ("SLICE_COLS", int(a[0].value[1:]), start, stop)
    if name == "LEFT" and len(a) == 2 and strcol(a[0]):
        return ("SLICE", int(a[0].value[1:]), 0, max(int_lit(a[1]), 0), 1)
    if name == "RIGHT" and len(a) == 2 and strcol(a[0]):
        k = max(int_lit(a[1]), 0)
        return ("SLICE", int(a[0].value[1:]), -k, 0 if k < 1 else None, 1)
    if name == "REVERSE" and len(a) == 1 and strcol(a[0]):
        return ("SLICE", int(a[0].value[1:]), None, None, -1)
    if name in ("UPPER", "LOWER", "INITCAP") and len(a) == 1 and strcol(a[0]):
        return (name, int(a[0].value[1:]))
    if name == "TRIM" and len(a) == 3 and strcol(a[2]):
        return ("TRIM", int(a[2].value[1:]), _unquote(a[0].value), _unquote(a[1].value))
    if name == "REPLACE" and len(a) == 3 and strcol(a[0]):
        return ("REPLACE", int(a[0].value[1:]), _unquote(a[1].value), _unquote(a[2].value))
    if name == "REGEXP_REPLACE" and len(a) in (3, 4) and strcol(a[0]) and _is_lit(a[1]) and _is_lit(a[2]):
        # LogicalProject.cpp:149-183: a position (1-based) keeps the characters before it
        start = int_lit(a[3]) - 1 if len(a) == 4 else 0
        if start < 0:
            raise ValueError("Position must be greater than zero.")
        return ("REGEX", int(a[0].value[1:]), _unquote(a[1].value), _unquote(a[2].value), start)
    if name in ("CONCAT", "||") and len(a) == 2:
        def operand(x):
            if strcol(x):
                return ("col", int(x.value[1:]))
            if _is_lit(x):
                return ("lit", _unquote(x.value))
            raise ValueError("CONCAT of something other than strings")
        return ("CONCAT", operand(a[0]), operand(a[1]))
    if name in ("CAST_VARCHAR", "CAST_CHAR") and len(a) == 1 and (a[0].var or a[0].op):
        return ("TO_STRING", int(a[0].value[1:]) if a[0].var else rebuild(a[0], typed=True))
    if name in PARSE_TYPES and len(a) == 1 and strcol(a[0]):
        t = PARSE_TYPES[name]
        fmt = None if t in (T.INT8, T.INT16, T.INT32, T.INT64, T.FLOAT32, T.FLOAT64) else \
            ("%Y-%m-%d" if t == T.TIMESTAMP_DAYS else "%Y-%m-%d %H:%M:%S")
        return ("PARSE", int(a[0].value[1:]), t, fmt)
    if name in ("TO_DATE", "TO_TIMESTAMP") and len(a) == 2 and strcol(a[0]) and _is_lit(a[1]):
        return ("PARSE", int(a[0].value[1:]), T.TIMESTAMP_DAYS if name == "TO_DATE" else T.TIMESTAMP_NANOSECONDS,
                _unquote(a[1].value))
    return None


def _regex(pattern: str):
    """REGEXP_REPLACE's pattern as a Python regular expression with the same
    leftmost-first semantics: ASCII classes and word boundaries (re.ASCII),
    `$` only at the end of the subject (Python's `$` also matches before a
    final newline, so it becomes `\\Z`).  Python's own backtracking matcher
    tries alternatives and repeats in the same order as the device's Pike VM."""
    out, i, n = [], 0, len(pattern)
    while i < n:
        c = pattern[i]
        if c == "\\" and i + 1 < n:
            out.append(pattern[i:i + 2])
            i += 2
        elif c == "[":  # copied up to its closing bracket (a ']' first is literal)
            j = i + 1
            if j < n and pattern[j] == "^":
                j += 1
            if j < n and pattern[j] == "]":
                j += 1
            while j < n and pattern[j] != "]":
                j += 2 if pattern[j] == "\\" else 1
            out.append(pattern[i:j + 1])
            i = j + 1
        else:
            out.append("\\Z" if c == "$" else c)
            i += 1
    return re.compile("".join(out), re.ASCII)


def _template(repl: str):
    """The replacement as parts: text, or a group number (\\N or ${N})."""
    parts, i = [], 0
    while i < len(repl):
        m = re.match(r"\\([0-9])|\$\{([0-9]+)\}", repl[i:])
        if m:
            parts.append(int(m.group(1) or m.group(2)))
            i += m.end()
        else:
            parts.append(repl[i])
            i += 1
    return parts


def _regex_replace(rx, tmpl, v: str) -> str:
    """Every (non-empty, non-overlapping) match, left to right, replaced by the
    template; a group that did not take part gives the empty string."""
    out, pos = [], 0
    for m in rx.finditer(v):
        out.append(v[pos:m.start()])
        out.extend(p if isinstance(p, str) else (m.group(p) or "") for p in tmpl)
        pos = m.end()
    out.append(v[pos:])
    return "".join(out)


def _slice_cols(v: str, start: int, stop: int) -> str:
    """cudf::strings::slice_strings with a start and a stop per row: the start
    clamped at 0, a stop below 0 or past the end meaning the end, empty when
    the start is not before the stop."""
    L = len(v)
    b = max(start, 0)
    if b >= L:
        return ""
    e = L if stop < 0 or stop > L else stop
    return v[b:e] if b < e else ""


# Powers of ten for scaling a double into [1, 10) by the binary decomposition
# of its decimal exponent (cudf::strings::from_floats' normalisation).
_SCALE = ((256, 1e256, 1e-255), (128, 1e128, 1e-127), (64, 1e64, 1e-63), (32, 1e32, 1e-31), (16, 1e16, 1e-15),
          (8, 1e8, 1e-7), (4, 1e4, 1e-3), (2, 1e2, 1e-1), (1, 1e1, 1e0))


def format_float(x: float) -> str:
    """CAST of a FLOAT64 (FLOAT32 widened) to VARCHAR as cudf::strings::from_floats
    writes it: values in [1e-4, 1e9) in fixed notation, others as d.ddd with a
    signed exponent of at least two digits; 9 significant digits at most (the
    integer part's digits take from the 9 decimal places), the last one rounded
    half up from the scaled remainder, trailing zeros dropped, at least one
    decimal place; NaN, Inf, -Inf.  Pinned by process_project.cpp:389-412."""
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "-Inf" if x < 0 else "Inf"
    neg = math.copysign(1.0, x) < 0
    v = abs(float(x))
    if v == 0.0:
        return "-0.0" if neg else "0.0"
    exp10 = 0
    if v >= 1e9:
        for fx, p, _ in _SCALE:
            if v >= p:
                v = v / p
                exp10 += fx
    elif v < 1e-4:
        for fx, p, lo in _SCALE:
            if v < lo:
                v = v * p
                exp10 -= fx
    whole = int(v)
    places, width = 9, 10 ** 9
    i = whole
    while i >= 10:
        places -= 1
        width //= 10
        i //= 10
    frac = (v - float(whole)) * float(width)
    dec = int(frac)
    dec += int(2.0 * (frac - float(dec)))
    if dec >= width:
        dec = 0
        whole += 1
        if exp10 and whole >= 10:
            exp10 += 1
            whole = 1
    while dec % 10 == 0 and places > 0:
        dec //= 10
        places -= 1
    out = ("-" if neg else "") + str(whole) + "." + (str(dec).zfill(places) if places > 0 else "0")
    if exp10:
        out += "e" + ("-" if exp10 < 0 else "+") + str(abs(exp10)).zfill(2)
    return out


def parse_float(v: str) -> float:
    """CAST of a string to FLOAT64 as cudf::strings::to_floats reads it: an
    optional sign, NaN / Inf / Infinity, else digits with one optional decimal
    point and an optional e / E exponent; up to 19 significant digits are
    accumulated into an integer (later ones only move the exponent), which is
    then scaled by exact powers of ten (divided for a negative exponent, in
    steps of 1e22), so that up to 15 digits and |exponent| <= 22 convert
    exactly rounded.  Anything else reads as the digits before it (0 for
    none).  Pinned by process_project.cpp:414-445."""
    i, n = 0, len(v)
    neg = False
    if i < n and v[i] in "+-":
        neg = v[i] == "-"
        i += 1
    rest = v[i:]
    if rest.startswith("NaN"):
        return math.nan
    if rest.startswith("Inf"):
        return -math.inf if neg else math.inf
    mant, digits, exp10, dot = 0, 0, 0, False
    while i < n:
        c = v[i]
        if c == "." and not dot:
            dot = True
        elif "0" <= c <= "9":
            if digits < 19:
                mant = mant * 10 + (ord(c) - 48)
                if mant:
                    digits += 1
                if dot:
                    exp10 -= 1
            elif not dot:
                exp10 += 1
        else:
            break
        i += 1
    if i < n and v[i] in "eE":
        j, eneg, e = i + 1, False, 0
        if j < n and v[j] in "+-":
            eneg = v[j] == "-"
            j += 1
        while j < n and "0" <= v[j] <= "9":
            e = min(e * 10 + (ord(v[j]) - 48), 100000)
            j += 1
        exp10 += -e if eneg else e
    x = float(mant)
    if exp10 >= 0:
        while exp10 > 22:
            x = x * 1e22
            exp10 -= 22
        x = x * float(10 ** exp10)
    else:
        e = -exp10
        while e > 22:
            x = x / 1e22
            e -= 22
        x = x / float(10 ** e)
    return -x if neg else x


def _slice(v: str, start, stop, step):
    """cudf::strings::slice_strings of one string, by characters."""
    L = len(v)
    if step < 0:
        return v[::-1]
    b = 0 if start is None else (min(start, L) if start >= 0 else max(L + start, 0))
    e = L if stop is None else (min(stop, L) if stop >= 0 else max(L + stop, 0))
    return v[b:e] if b < e else ""


def _upper(v: str) -> str:
    """UPPER per code point: its full uppercase mapping (SpecialCasing's
    unconditional entries included, e.g. U+00DF -> "SS"); no context rules."""
    return "".join(ch.upper() for ch in v)


def _lower(v: str) -> str:
    """LOWER per code point (so no final-sigma rule)."""
    return "".join(ch.lower() for ch in v)


def _initcap(v: str) -> str:
    """INITCAP (cudf::strings::title): in each run of alphabetic characters
    (general category L*), the first upper-cased, the rest lower-cased."""
    out, word = [], False
    for ch in v:
        letter = ch.isalpha()
        out.append((ch.lower() if word else ch.upper()) if letter else ch)
        word = letter
    return "".join(out)


def _trim(v: str, side: str, chars: str) -> str:
    def strip_me(c):
        return ord(c) <= 32 if chars == "" else c in chars
    b, e = 0, len(v)
    if side != "TRAILING":
        while b < e and strip_me(v[b]):
            b += 1
    if side != "LEADING":
        while e > b and strip_me(v[e - 1]):
            e -= 1
    return v[b:e]


def _civil(days: int) -> Tuple[int, int, int]:
    import datetime
    d = datetime.date(1970, 1, 1) + datetime.timedelta(days=days)
    return d.year, d.month, d.day


def format_value(t: int, x) -> str:
    """cast_to_str_functor for one valid value."""
    if t == T.BOOL8:
        return "true" if x else "false"
    if t in (T.FLOAT32, T.FLOAT64):
        return format_float(float(x))
    if t in (T.INT8, T.INT16, T.INT32, T.INT64, T.UINT8, T.UINT16, T.UINT32, T.UINT64):
        return str(int(x))
    if t == T.TIMESTAMP_DAYS:
        y, m, d = _civil(int(x))
        return f"{y:04d}-{m:02d}-{d:02d}"
    per = {T.TIMESTAMP_SECONDS: 1, T.TIMESTAMP_MILLISECONDS: 1000, T.TIMESTAMP_MICROSECONDS: 10 ** 6,
           T.TIMESTAMP_NANOSECONDS: 10 ** 9}[t]
    secs = int(x) // per
    days, sod = secs // 86400, secs % 86400
    y, m, d = _civil(days)
    return f"{y:04d}-{m:02d}-{d:02d} {sod // 3600:02d}:{sod // 60 % 60:02d}:{sod % 60:02d}"


def _digits(b: bytes) -> int:
    v = 0
    for c in b:
        if not 48 <= c <= 57:
            break
        v = v * 10 + c - 48
    return v


def _days_from_civil(y: int, m: int, d: int) -> int:
    y -= m <= 2
    era = (y if y >= 0 else y - 399) // 400
    yoe = y - era * 400
    doy = (153 * (m + (-3 if m > 2 else 9)) + 2) // 5 + d - 1
    doe = yoe * 365 + yoe // 4 - yoe // 100 + doy
    return era * 146097 + doe - 719468


def _format_items(fmt: str):
    """to_timestamps' items: (field index in Y m d H M S or None, width)."""
    items, i = [], 0
    while i < len(fmt):
        if fmt[i] == "%" and i + 1 < len(fmt):
            c = fmt[i + 1]
            i += 2
            items.append(("YmdHMS".index(c), 4 if c == "Y" else 2) if c != "%" else (None, 1))
        else:
            items.append((None, 1))
            i += 1
    return items


def parse_value(t: int, v: str, fmt: Optional[str] = None) -> int:
    """to_integers / to_timestamps of one valid string."""
    if t in (T.FLOAT32, T.FLOAT64):
        return parse_float(v)
    b = v.encode("utf-8")
    if t in (T.INT8, T.INT16, T.INT32, T.INT64):
        neg = b[:1] == b"-"
        x = _digits(b[1:] if b[:1] in (b"-", b"+") else b)
        x = (-x if neg else x) % (1 << 64)
        bits = {T.INT8: 8, T.INT16: 16, T.INT32: 32, T.INT64: 64}[t]
        x %= 1 << bits
        return x - (1 << bits) if x >= 1 << (bits - 1) else x

    f, at = [0] * 6, 0
    for field, width in _format_items(fmt or ("%Y-%m-%d" if t == T.TIMESTAMP_DAYS else "%Y-%m-%d %H:%M:%S")):
        w = max(0, min(width, len(b) - at))
        if field is not None:
            f[field] = _digits(b[at:at + w])
        at += w
    days = _days_from_civil(f[0], f[1], f[2])
    if t == T.TIMESTAMP_DAYS:
        return days
    secs = days * 86400 + f[3] * 3600 + f[4] * 60 + f[5]
    return secs * {T.TIMESTAMP_SECONDS: 1, T.TIMESTAMP_MILLISECONDS: 1000, T.TIMESTAMP_MICROSECONDS: 10 ** 6,
                   T.TIMESTAMP_NANOSECONDS: 10 ** 9}[t]


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
        elif op[0] in ("SLICE", "UPPER", "LOWER", "INITCAP", "TRIM", "REPLACE"):
            src = strings[op[1]]
            f = {"SLICE": lambda v: _slice(v, op[2], op[3], op[4]), "UPPER": _upper,
                 "LOWER": _lower, "INITCAP": _initcap,
                 "TRIM": lambda v: _trim(v, op[2], op[3]), "REPLACE": lambda v: v.replace(op[2], op[3])}[op[0]]
            strings[k] = [None if v is None else f(v) for v in src]
            table.append(HostColumn(T.INT8, np.zeros(n, dtype=np.int8)))
        elif op[0] == "REGEX":
            rx, tmpl = _regex(op[2]), _template(op[3])
            strings[k] = [None if v is None else v[:op[4]] + _regex_replace(rx, tmpl, v[op[4]:]) for v in strings[op[1]]]
            table.append(HostColumn(T.INT8, np.zeros(n, dtype=np.int8)))
        elif op[0] == "SLICE_COLS":
            def positions(text, default):
                if text is None:
                    return [default] * n
                c = pyoracle.evaluate_expressions(table, [text], nthreads)[0]
                valid = unpack_validity(c.mask, n) if c.mask is not None else np.ones(n, dtype=bool)
                return [int(c.data[i]) if valid[i] else 0 for i in range(n)]  # NULL positions read 0
            b0, e0 = positions(op[2], 0), positions(op[3], 2 ** 31 - 1)
            src = strings[op[1]]
            strings[k] = [None if v is None else _slice_cols(v, b0[i], e0[i]) for i, v in enumerate(src)]
            table.append(HostColumn(T.INT8, np.zeros(n, dtype=np.int8)))
        elif op[0] == "CONCAT":
            def side(o):
                return strings[o[1]] if o[0] == "col" else [o[1]] * n
            l, r = side(op[1]), side(op[2])
            strings[k] = [None if x is None or y is None else x + y for x, y in zip(l, r)]
            table.append(HostColumn(T.INT8, np.zeros(n, dtype=np.int8)))
        elif op[0] == "TO_STRING":
            if isinstance(op[1], int) and op[1] in strings:
                strings[k] = list(strings[op[1]])
            else:
                c = table[op[1]] if isinstance(op[1], int) else pyoracle.evaluate_expressions(table, [op[1]], nthreads)[0]
                valid = unpack_validity(c.mask, n) if c.mask is not None else np.ones(n, dtype=bool)
                strings[k] = [format_value(c.type_id, c.data[i]) if valid[i] else None for i in range(n)]
            table.append(HostColumn(T.INT8, np.zeros(n, dtype=np.int8)))
        elif op[0] == "PARSE":
            src, t = strings[op[1]], op[2]
            valid = np.array([v is not None for v in src])
            from blazingsql_gb300.types import np_dtype
            data = np.array([parse_value(t, v, op[3]) if v is not None else 0 for v in src], dtype=np_dtype(t))
            table.append(HostColumn(t, data, pack_validity(valid)))
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
