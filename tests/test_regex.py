"""REGEXP_REPLACE (LogicalProject.cpp:149-183): the pattern compiler and the
Pike VM matcher against the oracle (Python's re with the same leftmost-first
semantics), on the host through a host build of the same sources, and on the
GPU through the string pre-pass."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import strings_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PATTERNS = [
    "a", "ab|cd", "a+", "a+?", "(a|ab)(c|bcd)(d*)", "[a-c]+", "[^a-c ]+", r"\d+", r"\w+@\w+\.com", r"\s+",
    "^ab", "b$", r"\bab\b", r"\Bb", "(x)(y)?z", "é+", "[éà]x?", ".b", "a{2}", "a{1,3}", "a{2,}", "a{,2}b",
    "(?:ab)+", "(a)|b", "x*y", "colou?r", r"[\d.]+", "[]a]", "[a-]+", "(a|b)*?c", "(ab|a)(bc|c)?", r"\.",
    r"[\w-]+", r"\S+", r"\D", r"[^\d\s]+", "a.c", "(é)(.)", "[a-cx-z]{2,3}?", "d|c|b|a",
]
TEMPLATES = ["X", "", r"<\1>", r"${1}-\0", r"\0\0", "\\", "$", "é", r"[\2]", "${0}!"]
ALPHABET = list("abcdxyz é.@_-0 \n") + ["à", "colour", "color", "ab", "com"]


def _subjects(rng, n):
    out = ["", "a", "ab", "abcd", "aaab", "x@y.com a@b.com", "colour color", "abab ab", "é éé", "a\nb",
           "aab  bcd", "12.5 x 3"]
    while len(out) < n:
        out.append("".join(rng.choice(ALPHABET, int(rng.integers(0, 9)))))
    return out


def _expected(pattern, template, subject, keep=0):
    return subject[:keep] + strings_ref._regex_replace(strings_ref._regex(pattern), strings_ref._template(template),
                                                         subject[keep:])


def _groups(pattern):
    import re
    return re.compile(pattern).groups


@pytest.fixture(scope="module")
def host_regex(tmp_path_factory):
    """The compiler and matcher built for the host from the device sources."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("regex") / "libregex_host.so")
    subprocess.run([cxx, "-O1", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "blazingsql_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "regex_vm_host.cpp"), "-o", out], check=True)
    lib = C.CDLL(out)
    f = lib.gx_test_regex_replace
    f.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_char_p, C.c_int, C.c_char_p, C.c_int]
    f.restype = C.c_int

    def run(pattern, template, subject, keep=0):
        b = subject.encode()
        buf, err = C.create_string_buffer(4096), C.create_string_buffer(512)
        n = f(pattern.encode(), template.encode(), b, len(b), keep, buf, 4096, err, 512)
        if n < 0:
            raise ValueError(err.value.decode())
        return buf.raw[:n].decode()
    return run


def test_regex_host_matches_oracle(host_regex):
    rng = np.random.default_rng(7)
    subjects = _subjects(rng, 60)
    checked = 0
    for p in PATTERNS:
        for t in TEMPLATES:
            if any(f"\\{g}" in t or f"${{{g}}}" in t for g in range(_groups(p) + 1, 10)):
                continue  # refers to a group the pattern lacks
            for s in subjects:
                assert host_regex(p, t, s) == _expected(p, t, s), (p, t, s)
                checked += 1
    assert checked > 10_000


def test_regex_host_position(host_regex):
    for s in ["aaaa", "abab", "é a é a", "", "ab"]:
        for keep in range(0, 6):
            assert host_regex("a", "X", s, keep) == _expected("a", "X", s, keep), (s, keep)
            assert host_regex("^a", "X", s, keep) == _expected("^a", "X", s, keep), (s, keep)
            assert host_regex(r"\ba", "X", s, keep) == _expected(r"\ba", "X", s, keep), (s, keep)


@pytest.mark.parametrize("pattern", ["", "a*", "(a*)+", "a**", "(?=a)", r"\1", "a{2,1}", "(", ")", "[a", "x{",
                                     r"\p", "^", r"\b", "a|", "*a", "(?i)a", "a{1001}", "(ab){40}"])
def test_regex_host_rejects(host_regex, pattern):
    with pytest.raises(ValueError, match="REGEXP_REPLACE"):
        host_regex(pattern, "X", "abc")


def test_regex_host_template_errors(host_regex):
    with pytest.raises(ValueError, match="group 2"):
        host_regex("(a)", r"\2", "a")
    with pytest.raises(ValueError, match="above 4"):
        host_regex("(a)(b)(c)(d)(e)", r"\5", "abcde")
    assert host_regex("(a)(b)(c)(d)(e)", r"\4", "abcde") == "d"  # groups past 4 may exist unreferenced


REGEX_EXPRS = [
    "REGEXP_REPLACE($0, 'a+', 'X')",
    "REGEXP_REPLACE($0, '(a|b)(c)?', '[\\2\\1]')",
    "REGEXP_REPLACE($0, '[^a-c]', '')",
    "REGEXP_REPLACE($0, '\\w+@(\\w+)\\.com', '<${1}>')",
    "REGEXP_REPLACE($0, 'é|à', 'E')",
    "REGEXP_REPLACE($0, '^.', '#')",
    "REGEXP_REPLACE($0, '.$', '#')",
    "REGEXP_REPLACE($0, 'b', 'Y', 3)",
    "REGEXP_REPLACE($0, '^b', 'Y', 2)",
    "CHAR_LENGTH(REGEXP_REPLACE($0, 'a', 'aa'))",
    "REGEXP_REPLACE(UPPER($1), 'A+', '-')",
]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 33, 5000, 70_001])
def test_regex_replace_gpu(n):
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    from blazingsql_gb300.types import HostColumn, TypeId as T
    rng = np.random.default_rng(900 + n)
    s0 = [None if rng.random() < 0.1 else v for v in _subjects(rng, n)][:n]
    s1 = ["".join(rng.choice(list("abAB c"), int(rng.integers(0, 7)))) for _ in range(n)]
    cols = [None, None, HostColumn(T.INT64, np.arange(n, dtype=np.int64))]
    strings = {0: s0, 1: s1}
    dev = [DeviceColumn.from_strings(s0), DeviceColumn.from_strings(s1), DeviceColumn.from_host(cols[2])]
    got = g.evaluate_expressions(dev, REGEX_EXPRS)
    exp = strings_ref.evaluate_expressions(cols, strings, REGEX_EXPRS)
    for i, (a, e) in enumerate(zip(got, exp)):
        a = a.to_strings() if a.type_id == T.STRING else a.to_host()
        if isinstance(e, list):
            assert a == e, (REGEX_EXPRS[i], a[:8], e[:8])
        else:
            assert np.array_equal(a.values()[e.valid()], e.values()[e.valid()]), REGEX_EXPRS[i]
            assert np.array_equal(a.valid(), e.valid()), REGEX_EXPRS[i]


@pytest.mark.gpu
def test_regex_replace_gpu_errors():
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    from blazingsql_gb300.api import DeviceColumn
    dev = [DeviceColumn.from_strings(["ab", "b"])]
    with pytest.raises(N.GxError, match="empty string"):
        g.evaluate_expressions(dev, ["REGEXP_REPLACE($0, 'a*', 'X')"])
    with pytest.raises(N.GxError, match="greater than zero"):
        g.evaluate_expressions(dev, ["REGEXP_REPLACE($0, 'a', 'X', 0)"])
    with pytest.raises(N.GxError, match="occurrence"):
        g.evaluate_expressions(dev, ["REGEXP_REPLACE($0, 'a', 'X', 1, 1)"])
    with pytest.raises(N.GxError, match="group 1"):
        g.evaluate_expressions(dev, ["REGEXP_REPLACE($0, 'a', '\\1')"])
