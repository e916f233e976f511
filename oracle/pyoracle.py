"""ctypes front for the CPU oracle (test infrastructure only).

Loaded by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg as
the checker; the product (``blazingsql_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import List, Sequence, Tuple

import numpy as np

from blazingsql_gb300.types import HostColumn, np_dtype

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgx_oracle.so")
_lib = None


class OracleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class _Col(C.Structure):
    _fields_ = [("type_id", C.c_int32), ("pad_", C.c_int32), ("data", C.c_void_p),
                ("null_mask", C.c_void_p), ("offset", C.c_int64), ("size", C.c_int64)]


class _Out(C.Structure):
    _fields_ = [("type_id", C.c_int32), ("pad_", C.c_int32), ("data", C.c_void_p),
                ("null_mask", C.c_void_p), ("size", C.c_int64)]


def build() -> str:
    """Compile the oracle with its Makefile (g++); returns the library path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.oracle_evaluate_expressions.argtypes = [C.POINTER(_Col), C.c_int, C.POINTER(C.c_char_p), C.c_int,
                                                  C.POINTER(_Out), C.c_int, C.c_uint64, C.c_char_p, C.c_int]
        L.oracle_process_filter.argtypes = [C.POINTER(_Col), C.c_int, C.c_char_p, C.POINTER(_Out),
                                            C.POINTER(C.c_int64), C.c_int, C.c_char_p, C.c_int]
        L.oracle_process_project.argtypes = [C.POINTER(_Col), C.c_int, C.c_char_p, C.POINTER(_Out), C.c_int,
                                             C.POINTER(C.c_int), C.c_int, C.c_uint64, C.c_char_p, C.c_int]
        L.oracle_filter_project.argtypes = [C.POINTER(_Col), C.c_int, C.c_char_p, C.POINTER(C.c_char_p), C.c_int,
                                            C.POINTER(_Out), C.POINTER(C.c_int64), C.c_int, C.c_uint64,
                                            C.c_char_p, C.c_int]
        L.oracle_rebuild_expression.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        L.oracle_string_transform.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
        L.oracle_round_scale.argtypes = [C.c_double]
        L.oracle_round_scale.restype = C.c_double
        L.oracle_philox_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64]
        L.oracle_philox_uniform.restype = C.c_double
        L.oracle_free_columns.argtypes = [C.POINTER(_Out), C.c_int]
        _lib = L
    return _lib


def _cols(cols: Sequence[HostColumn]):
    arr = (_Col * max(1, len(cols)))()
    for i, c in enumerate(cols):
        arr[i].type_id = c.type_id
        arr[i].data = c.data.ctypes.data
        arr[i].null_mask = c.mask.ctypes.data if c.mask is not None else None
        arr[i].offset = c.offset
        arr[i].size = c.size
    return arr


def _take(outs, n: int) -> List[HostColumn]:
    res = []
    for i in range(n):
        o = outs[i]
        dt = np_dtype(o.type_id)
        size = int(o.size)
        data = np.ctypeslib.as_array(C.cast(o.data, C.POINTER(C.c_uint8)), shape=(max(1, size) * dt.itemsize,))
        data = data[:size * dt.itemsize].view(dt).copy()
        nwords = max(16, ((size + 31) // 32 + 15) // 16 * 16)
        mask = np.ctypeslib.as_array(C.cast(o.null_mask, C.POINTER(C.c_uint32)), shape=(nwords,)).copy()
        res.append(HostColumn(o.type_id, data, mask))
    lib().oracle_free_columns(outs, n)
    return res


def _check(rc: int, err) -> None:
    if rc != 0:
        raise OracleError(rc, err.value.decode(errors="replace"))


def evaluate_expressions(cols: Sequence[HostColumn], exprs: Sequence[str], nthreads: int = 1,
                         seed: int = 0) -> List[HostColumn]:
    L = lib()
    err = C.create_string_buffer(1024)
    ex = (C.c_char_p * len(exprs))(*[e.encode() for e in exprs])
    outs = (_Out * max(1, len(exprs)))()
    _check(L.oracle_evaluate_expressions(_cols(cols), len(cols), ex, len(exprs), outs, nthreads, seed, err, 1024), err)
    return _take(outs, len(exprs))


def process_filter(cols: Sequence[HostColumn], query_part: str, nthreads: int = 1) -> List[HostColumn]:
    L = lib()
    err = C.create_string_buffer(1024)
    outs = (_Out * max(1, len(cols)))()
    rows = C.c_int64(0)
    _check(L.oracle_process_filter(_cols(cols), len(cols), query_part.encode(), outs, C.byref(rows), nthreads,
                                   err, 1024), err)
    return _take(outs, len(cols))


def process_project(cols: Sequence[HostColumn], query_part: str, nthreads: int = 1,
                    seed: int = 0) -> List[HostColumn]:
    L = lib()
    err = C.create_string_buffer(1024)
    outs = (_Out * 256)()
    n = C.c_int(0)
    _check(L.oracle_process_project(_cols(cols), len(cols), query_part.encode(), outs, 256, C.byref(n), nthreads,
                                    seed, err, 1024), err)
    return _take(outs, n.value)


def filter_project(cols: Sequence[HostColumn], condition: str, exprs: Sequence[str], nthreads: int = 1,
                   seed: int = 0) -> Tuple[List[HostColumn], int]:
    L = lib()
    err = C.create_string_buffer(1024)
    ex = (C.c_char_p * len(exprs))(*[e.encode() for e in exprs])
    outs = (_Out * max(1, len(exprs)))()
    rows = C.c_int64(0)
    _check(L.oracle_filter_project(_cols(cols), len(cols), condition.encode(), ex, len(exprs), outs, C.byref(rows),
                                   nthreads, seed, err, 1024), err)
    return _take(outs, len(exprs)), rows.value


def rebuild_expression(expr: str) -> str:
    buf = C.create_string_buffer(4096)
    rc = lib().oracle_rebuild_expression(expr.encode(), buf, 4096)
    if rc != 0:
        raise OracleError(rc, buf.value.decode())
    return buf.value.decode()


def string_transform(which: str, s: str) -> str:
    buf = C.create_string_buffer(8192)
    rc = lib().oracle_string_transform(which.encode(), s.encode(), buf, 8192)
    if rc != 0:
        raise OracleError(rc, buf.value.decode())
    return buf.value.decode()


def round_scale(d: float) -> float:
    return lib().oracle_round_scale(d)


def philox_uniform(seed: int, rand_id: int, row: int) -> float:
    return lib().oracle_philox_uniform(seed, rand_id, row)
