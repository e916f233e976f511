"""Column types and host-side column containers.

Type ids follow ``cudf::type_id`` as of cudf 21.08, the layout BlazingSQL's
evaluator consumes (``engine/src/Interpreter/interpreter_ops.cuh`` reads columns
through ``cudf::column_device_view``).  Validity masks are Arrow-style: ``uint32``
words, bit ``r % 32`` of word ``r // 32`` is row ``r``, 1 = valid.
"""
from __future__ import annotations

import enum
from dataclasses import dataclass
from typing import Optional

import numpy as np


class TypeId(enum.IntEnum):
    EMPTY = 0
    INT8 = 1
    INT16 = 2
    INT32 = 3
    INT64 = 4
    UINT8 = 5
    UINT16 = 6
    UINT32 = 7
    UINT64 = 8
    FLOAT32 = 9
    FLOAT64 = 10
    BOOL8 = 11
    TIMESTAMP_DAYS = 12
    TIMESTAMP_SECONDS = 13
    TIMESTAMP_MILLISECONDS = 14
    TIMESTAMP_MICROSECONDS = 15
    TIMESTAMP_NANOSECONDS = 16
    DURATION_DAYS = 17
    DURATION_SECONDS = 18
    DURATION_MILLISECONDS = 19
    DURATION_MICROSECONDS = 20
    DURATION_NANOSECONDS = 21
    DICTIONARY32 = 22
    STRING = 23


_NP = {
    TypeId.INT8: np.int8, TypeId.INT16: np.int16, TypeId.INT32: np.int32, TypeId.INT64: np.int64,
    TypeId.UINT8: np.uint8, TypeId.UINT16: np.uint16, TypeId.UINT32: np.uint32, TypeId.UINT64: np.uint64,
    TypeId.FLOAT32: np.float32, TypeId.FLOAT64: np.float64, TypeId.BOOL8: np.uint8,
    TypeId.TIMESTAMP_DAYS: np.int32, TypeId.TIMESTAMP_SECONDS: np.int64, TypeId.TIMESTAMP_MILLISECONDS: np.int64,
    TypeId.TIMESTAMP_MICROSECONDS: np.int64, TypeId.TIMESTAMP_NANOSECONDS: np.int64,
    TypeId.DURATION_DAYS: np.int32, TypeId.DURATION_SECONDS: np.int64, TypeId.DURATION_MILLISECONDS: np.int64,
    TypeId.DURATION_MICROSECONDS: np.int64, TypeId.DURATION_NANOSECONDS: np.int64,
}


def np_dtype(t: int) -> np.dtype:
    """numpy storage dtype of a fixed-width column type."""
    return np.dtype(_NP[TypeId(t)])


def is_float(t: int) -> bool:
    return int(t) in (TypeId.FLOAT32, TypeId.FLOAT64)


def pack_validity(valid: np.ndarray) -> np.ndarray:
    """bool[n] -> uint32 words (LSB = lowest row), padded to 16 words (64 B)."""
    valid = np.asarray(valid, dtype=bool)
    n = valid.shape[0]
    nwords = (n + 31) // 32
    padded_words = max(16, (nwords + 15) // 16 * 16)
    bits = np.zeros(padded_words * 32, dtype=np.uint8)
    bits[:n] = valid
    return np.packbits(bits, bitorder="little").view(np.uint32).copy()


def unpack_validity(mask: Optional[np.ndarray], n: int, offset: int = 0) -> np.ndarray:
    """uint32 words -> bool[n] for rows [offset, offset + n)."""
    if mask is None:
        return np.ones(n, dtype=bool)
    bits = np.unpackbits(np.asarray(mask, dtype=np.uint32).view(np.uint8), bitorder="little")
    return bits[offset:offset + n].astype(bool)


@dataclass
class HostColumn:
    """A fixed-width column in host memory (numpy), optionally nullable."""
    type_id: int
    data: np.ndarray
    mask: Optional[np.ndarray] = None   # uint32 words or None (all valid)
    offset: int = 0
    size: int = -1

    def __post_init__(self):
        self.type_id = int(self.type_id)
        self.data = np.ascontiguousarray(self.data, dtype=np_dtype(self.type_id))
        if self.mask is not None:
            self.mask = np.ascontiguousarray(self.mask, dtype=np.uint32)
        if self.size < 0:
            self.size = self.data.shape[0] - self.offset

    @staticmethod
    def from_values(type_id: int, values, valid=None) -> "HostColumn":
        data = np.asarray(values).astype(np_dtype(type_id))
        mask = None if valid is None else pack_validity(np.asarray(valid, dtype=bool))
        return HostColumn(type_id, data, mask)

    def valid(self) -> np.ndarray:
        return unpack_validity(self.mask, self.size, self.offset)

    def values(self) -> np.ndarray:
        return self.data[self.offset:self.offset + self.size]
