"""Host-side mirror of BlazingSQL's evaluator interface over the C ABI.

Names and argument meaning follow the reference:
``evaluate_expressions(table, expressions)`` (LogicalProject.cpp:796),
``process_project(table, query_part)`` (LogicalProject.cpp:943) and
``process_filter(table, query_part)`` (LogicalFilter.cpp:31).  Errors surface
as :class:`GxError` with the C status code (``retryable`` for OOM, as the
reference maps ``rmm::bad_alloc`` to a retry).

Device memory for inputs is held by torch tensors (plain device buffers);
outputs are owned by the native library and released when the returned
:class:`NativeColumn` objects are garbage collected.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _native as N
from .types import HostColumn, TypeId, np_dtype, pack_validity


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required (the evaluator has no CPU path)")
    return torch


def _stream_handle(stream) -> int:
    if stream is None:
        torch = _torch()
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


@dataclass
class DeviceColumn:
    """A borrowed device column: raw byte tensors for data and validity words."""
    type_id: int
    data: object                  # torch.uint8 tensor on the device (STRING: the characters)
    mask: Optional[object]        # torch.uint8 tensor (uint32 words) or None
    offset: int
    size: int
    str_offsets: Optional[object] = None  # STRING: torch.int32 tensor of size + 1 offsets

    @staticmethod
    def from_strings(values: Sequence[Optional[str]], device: str = "cuda") -> "DeviceColumn":
        """A STRING column (cudf layout: int32 offsets + UTF-8 characters);
        None entries are NULL."""
        torch = _torch()
        enc = [b"" if v is None else v.encode("utf-8") for v in values]
        offs = np.zeros(len(enc) + 1, dtype=np.int32)
        offs[1:] = np.cumsum([len(e) for e in enc])
        chars = np.frombuffer(b"".join(enc) or b"\0", dtype=np.uint8)
        mask = None
        if any(v is None for v in values):
            mask = torch.from_numpy(pack_validity(np.array([v is not None for v in values])).view(np.uint8)
                                    .copy()).to(device)
        return DeviceColumn(TypeId.STRING, torch.from_numpy(chars.copy()).to(device), mask, 0, len(values),
                            torch.from_numpy(offs).to(device))

    @staticmethod
    def from_host(col: HostColumn, device: str = "cuda") -> "DeviceColumn":
        torch = _torch()
        raw = np.ascontiguousarray(col.data).view(np.uint8)
        data = torch.from_numpy(raw.copy()).to(device) if raw.size else torch.zeros(64, dtype=torch.uint8,
                                                                                      device=device)
        mask = None
        if col.mask is not None:
            mask = torch.from_numpy(np.ascontiguousarray(col.mask).view(np.uint8).copy()).to(device)
        return DeviceColumn(col.type_id, data, mask, col.offset, col.size)

    def view(self) -> N.ColumnView:
        # cached per (tensors, offset, size): data_ptr() calls cost microseconds per batch
        key = (id(self.data), id(self.mask), self.offset, self.size, self.type_id, id(self.str_offsets))
        cached = getattr(self, "_view_cache", None)
        if cached is not None and cached[0] == key:
            return cached[1]
        v = N.ColumnView()
        v.type_id = self.type_id
        v.data = self.data.data_ptr()
        v.null_mask = self.mask.data_ptr() if self.mask is not None else None
        v.offset = self.offset
        v.size = self.size
        v.string_offsets = self.str_offsets.data_ptr() if self.str_offsets is not None else None
        self._view_cache = (key, v)
        return v


class NativeColumn:
    """An output column owned by the native library."""

    def __init__(self, col: N.Column, stream: int = 0):
        self._c = col
        self._stream = stream

    @property
    def type_id(self) -> int:
        return self._c.type_id

    @property
    def capacity(self) -> int:
        """Rows the column's buffers hold (at least size)."""
        return self._c.capacity

    @property
    def size(self) -> int:
        return self._c.size

    @property
    def data_ptr(self) -> int:
        return self._c.data or 0

    @property
    def mask_ptr(self) -> int:
        return self._c.null_mask or 0

    def view(self) -> N.ColumnView:
        v = N.ColumnView()
        v.type_id, v.data, v.null_mask, v.offset, v.size = self._c.type_id, self._c.data, self._c.null_mask, 0, \
            self._c.size
        v.string_offsets = self._c.string_offsets
        return v

    def to_strings(self) -> List[Optional[str]]:
        """A STRING column's rows (None where NULL)."""
        if self.type_id != TypeId.STRING:
            raise TypeError("not a string column")
        n = self.size
        offs = np.zeros(n + 1, dtype=np.int32)
        st = N.StatusInfo()
        N.check(N.lib().gx_string_offsets_to_host(C.byref(self._c), offs.ctypes.data, self._stream, C.byref(st)), st)
        chars = np.zeros(max(int(self._c.string_bytes), 1), dtype=np.uint8)
        nwords = max(16, ((n + 31) // 32 + 15) // 16 * 16)
        mask = np.zeros(nwords, dtype=np.uint32)
        N.check(N.lib().gx_column_to_host(C.byref(self._c), chars.ctypes.data, mask.ctypes.data, self._stream,
                                          C.byref(st)), st)
        raw = chars.tobytes()
        return [raw[offs[i]:offs[i + 1]].decode("utf-8") if (mask[i >> 5] >> (i & 31)) & 1 else None
                for i in range(n)]

    def to_host(self) -> HostColumn:
        if self.type_id == TypeId.STRING:
            raise TypeError("a string column: use to_strings()")
        dt = np_dtype(self.type_id)
        data = np.empty(max(self.size, 1), dtype=dt)
        nwords = max(16, ((self.size + 31) // 32 + 15) // 16 * 16)
        mask = np.zeros(nwords, dtype=np.uint32)
        st = N.StatusInfo()
        N.check(N.lib().gx_column_to_host(C.byref(self._c), data.ctypes.data, mask.ctypes.data, self._stream,
                                          C.byref(st)), st)
        return HostColumn(self.type_id, data[:self.size], mask)

    def free(self):
        if self._c.data:
            N.lib().gx_free_columns(C.byref(self._c), 1, self._stream)
            self._c.data = None
            self._c.null_mask = None
            self._c.string_offsets = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


Table = Sequence[Union[DeviceColumn, HostColumn, NativeColumn]]


def _views(table: Table, keep: list):
    cols = []
    for c in table:
        if isinstance(c, HostColumn):
            c = DeviceColumn.from_host(c)
        keep.append(c)
        cols.append(c.view())
    arr = (N.ColumnView * max(1, len(cols)))(*cols)
    return arr, len(cols)


def _wrap(outs, n: int, stream: int) -> List[NativeColumn]:
    return [NativeColumn(N.Column(outs[i].type_id, 0, outs[i].data, outs[i].null_mask, outs[i].size,
                                  outs[i].capacity, outs[i].string_offsets, outs[i].string_bytes), stream)
            for i in range(n)]


def evaluate_expressions(table: Table, expressions: Sequence[str], stream=None) -> List[NativeColumn]:
    """ral::processor::evaluate_expressions: one output column per expression."""
    keep: list = []
    views, nc = _views(table, keep)
    s = _stream_handle(stream)
    ex = (C.c_char_p * max(1, len(expressions)))(*[e.encode() for e in expressions])
    outs = (N.Column * max(1, len(expressions)))()
    st = N.StatusInfo()
    N.check(N.lib().gx_evaluate_expressions(views, nc, ex, len(expressions), outs, s, C.byref(st)), st)
    return _wrap(outs, len(expressions), s)


def process_project(table: Table, query_part: str, stream=None) -> Tuple[List[NativeColumn], List[str]]:
    """ral::processor::process_project on a LogicalProject(...) text."""
    keep: list = []
    views, nc = _views(table, keep)
    s = _stream_handle(stream)
    max_out = 256
    outs = (N.Column * max_out)()
    names = C.create_string_buffer(max_out * 128)
    nout = C.c_int(0)
    st = N.StatusInfo()
    N.check(N.lib().gx_process_project(views, nc, query_part.encode(), outs, max_out, C.byref(nout), names, 128, s,
                                       C.byref(st)), st)
    raw = names.raw
    out_names = [raw[i * 128:(i + 1) * 128].split(b"\0", 1)[0].decode() for i in range(nout.value)]
    return _wrap(outs, nout.value, s), out_names


def process_filter(table: Table, query_part: str, stream=None) -> List[NativeColumn]:
    """ral::processor::process_filter on a LogicalFilter(condition=[...]) text."""
    keep: list = []
    views, nc = _views(table, keep)
    s = _stream_handle(stream)
    outs = (N.Column * max(1, nc))()
    rows = C.c_int64(0)
    st = N.StatusInfo()
    N.check(N.lib().gx_process_filter(views, nc, query_part.encode(), outs, C.byref(rows), s, C.byref(st)), st)
    return _wrap(outs, nc, s)


def filter_project(table: Table, condition: Optional[str], expressions: Sequence[str],
                   stream=None) -> List[NativeColumn]:
    """process_project(process_filter(table, condition), expressions) in one device pass."""
    keep: list = []
    views, nc = _views(table, keep)
    s = _stream_handle(stream)
    ex = (C.c_char_p * len(expressions))(*[e.encode() for e in expressions])
    outs = (N.Column * len(expressions))()
    rows = C.c_int64(0)
    st = N.StatusInfo()
    cond = condition.encode() if condition else None
    N.check(N.lib().gx_filter_project(views, nc, cond, ex, len(expressions), outs, C.byref(rows), s, C.byref(st)),
            st)
    return _wrap(outs, len(expressions), s)


class Plan:
    """A compiled filter+project plan (gx_plan_compile / gx_plan_execute)."""

    def __init__(self, schema: Sequence[int], condition: Optional[str], expressions: Sequence[str],
                 nullable: Optional[Sequence[bool]] = None, filter_mode: int = N.GX_FILTER_AUTO,
                 block_threads: int = 0, words_per_warp: int = 0, short_circuit: bool = False,
                 conjunct_order: Optional[Sequence[int]] = None, rand_seed: int = 0):
        L = N.lib()
        o = N.PlanOptions()
        L.gx_plan_options_init(C.byref(o))
        o.filter_mode = filter_mode
        o.block_threads = block_threads
        o.words_per_warp = words_per_warp
        o.short_circuit = 1 if short_circuit else 0
        o.rand_seed = rand_seed
        if conjunct_order:
            o.num_conjuncts = len(conjunct_order)
            for i, c in enumerate(conjunct_order):
                o.conjunct_order[i] = c
        types = (C.c_int32 * max(1, len(schema)))(*[int(t) for t in schema])
        nb = None
        if nullable is not None:
            nb = (C.c_uint8 * max(1, len(schema)))(*[1 if x else 0 for x in nullable])
        ex = (C.c_char_p * max(1, len(expressions)))(*[e.encode() for e in expressions])
        st = N.StatusInfo()
        h = L.gx_plan_compile(types, nb, len(schema), condition.encode() if condition else None, ex,
                              len(expressions), C.byref(o), C.byref(st))
        if not h:
            raise N.GxError(st.code, st.message.decode(errors="replace"))
        self._h = h
        self.schema = list(schema)

    @property
    def num_outputs(self) -> int:
        return N.lib().gx_plan_num_outputs(self._h)

    @property
    def num_conjuncts(self) -> int:
        return N.lib().gx_plan_num_conjuncts(self._h)

    def output_types(self) -> List[int]:
        return [N.lib().gx_plan_output_type(self._h, i) for i in range(self.num_outputs)]

    def execute(self, table: Table, out: Optional[Sequence[N.Column]] = None, stream=None):
        """Runs the plan; returns (columns, rows).  ``out`` may hold caller buffers."""
        keep: list = []
        views, nc = _views(table, keep)
        s = _stream_handle(stream)
        n = self.num_outputs
        outs = (N.Column * max(1, n))()
        if out is not None:
            for i, c in enumerate(out):
                outs[i] = c
        rows = C.c_int64(0)
        st = N.StatusInfo()
        rc = N.lib().gx_plan_execute(self._h, views, nc, outs, C.byref(rows), s, C.byref(st))
        if rc == N.GX_ERR_CAPACITY:
            raise N.GxError(rc, f"{st.message.decode(errors='replace')} (needed rows={rows.value})")
        N.check(rc, st)
        if out is not None:
            return [outs[i] for i in range(n)], rows.value
        return _wrap(outs, n, s), rows.value

    def execute_host(self, columns, outputs, stream=None) -> int:
        """gx_plan_execute_host: host memory in, host memory out.

        ``columns``: one (type_id, data_ptr, mask_ptr or 0, rows) per input;
        ``outputs``: one (data_ptr, mask_ptr, capacity_rows) per output, all
        host addresses (numpy ``ctypes.data`` or pinned torch ``data_ptr()``).
        Returns the output row count."""
        nc = len(columns)
        views = (N.ColumnView * max(1, nc))()
        for i, (t, d, m, rows) in enumerate(columns):
            views[i].type_id = int(t)
            views[i].data = d
            views[i].null_mask = m or None
            views[i].offset = 0
            views[i].size = rows
        n = self.num_outputs
        outs = (N.Column * max(1, n))()
        for j, (d, m, cap) in enumerate(outputs):
            outs[j].data = d
            outs[j].null_mask = m
            outs[j].capacity = cap
        rows = C.c_int64(0)
        st = N.StatusInfo()
        rc = N.lib().gx_plan_execute_host(self._h, views, nc, outs, C.byref(rows), _stream_handle(stream),
                                          C.byref(st))
        if rc == N.GX_ERR_CAPACITY:
            raise N.GxError(rc, f"{st.message.decode(errors='replace')} (needed rows={rows.value})")
        N.check(rc, st)
        return rows.value

    def execute_noalloc(self, table: Table, out: Sequence[N.Column], stream=None):
        """gx_plan_execute_noalloc: runs the filter plan into the caller's buffers
        (``out``: one Column per output with data, null_mask and capacity set)
        without any device allocation by the library.  Returns (columns, rows)."""
        keep: list = []
        views, nc = _views(table, keep)
        s = _stream_handle(stream)
        outs = (N.Column * max(1, len(out)))(*out)
        rows = C.c_int64(0)
        st = N.StatusInfo()
        N.check(N.lib().gx_plan_execute_noalloc(self._h, views, nc, outs, C.byref(rows), s, C.byref(st)), st)
        return [outs[i] for i in range(len(out))], rows.value

    def wait_test(self, table: Table, first_tile: int, spin_limit: int) -> int:
        """gx_debug_filter_timeout: runs the plan with the tile ticket starting
        at ``first_tile`` and bounded waits of ``spin_limit`` polls; returns the
        status code (GX_ERR_TIMEOUT when a wait gave up)."""
        keep: list = []
        views, nc = _views(table, keep)
        st = N.StatusInfo()
        return N.lib().gx_debug_filter_timeout(self._h, views, nc, first_tile, spin_limit, C.byref(st))

    def kernel_source(self, kind: int = 1, has_mask: Optional[Sequence[bool]] = None) -> str:
        L = N.lib()
        st = N.StatusInfo()
        hm = None if has_mask is None else (C.c_uint8 * len(has_mask))(*[1 if x else 0 for x in has_mask])
        n = L.gx_debug_kernel_source(self._h, kind, hm, None, 0, C.byref(st))
        if n < 0:
            raise N.GxError(st.code, st.message.decode(errors="replace"))
        buf = C.create_string_buffer(n + 1)
        L.gx_debug_kernel_source(self._h, kind, hm, buf, n + 1, C.byref(st))
        return buf.value.decode()

    def resources(self, kind: int = 1, has_mask: Optional[Sequence[bool]] = None):
        """(registers, spill bytes, static shared bytes) of a plan kernel for sm_103a."""
        st = N.StatusInfo()
        hm = None if has_mask is None else (C.c_uint8 * len(has_mask))(*[1 if x else 0 for x in has_mask])
        r, sp, sh = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        N.check(N.lib().gx_debug_kernel_resources(self._h, kind, hm, C.byref(r), C.byref(sp), C.byref(sh),
                                                  C.byref(st)), st)
        return r.value, sp.value, sh.value

    def compile_check(self, kind: int = 1, has_mask: Optional[Sequence[bool]] = None) -> None:
        st = N.StatusInfo()
        hm = None if has_mask is None else (C.c_uint8 * len(has_mask))(*[1 if x else 0 for x in has_mask])
        N.check(N.lib().gx_debug_compile_check(self._h, kind, hm, C.byref(st)), st)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                N.lib().gx_plan_destroy(self._h)
                self._h = None
        except Exception:
            pass


class _Queue:
    """Arguments and result arrays of one gx_learner_execute_batches call."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


class _BatchReport(dict):
    """Per-batch report of the learner (a dict, filled on first access)."""

    def __init__(self, info):
        super().__init__()
        self._info = info

    def _fill(self):
        if self._info is None:
            return
        info, self._info = self._info, None
        k = info.num_conjuncts
        self.update({"path": info.path, "reruns": info.reruns, "rows": info.rows,
                     "predicted_rows": info.predicted_rows, "train_loss": info.train_loss,
                     "order": list(info.order[:k]), "predicted_sel": list(info.predicted_sel[:k]),
                     "measured_sel": list(info.measured_sel[:k])})

    def __getitem__(self, key):
        self._fill()
        return super().__getitem__(key)

    def __repr__(self):
        self._fill()
        return super().__repr__()


class BoundBatches:
    """A list of batches as one array of C column views (BatchRunner.bind)."""

    def __init__(self, views, count: int, keep: list):
        self.views = views
        self.count = count
        self._keep = keep


def free_column_array(outs, count: int, stream=None) -> None:
    """Releases `count` library-owned columns of a C array with one call."""
    if count > 0:
        N.lib().gx_free_columns(outs, count, _stream_handle(stream))


class BatchRunner:
    """A table of batches of one filter plan through one persistent kernel in a
    captured CUDA graph (gx_batch_runner_*)."""

    def __init__(self, plan: Plan, max_batches: int, max_total_rows: int, autotune: bool = True):
        st = N.StatusInfo()
        h = N.lib().gx_batch_runner_create(plan._h, max_batches, max_total_rows, 1 if autotune else 0, C.byref(st))
        if not h:
            raise N.GxError(st.code, st.message.decode(errors="replace"))
        self._h = h
        self.num_outputs = plan.num_outputs
        self._ncols = len(plan.schema)

    def bind(self, batches: Sequence[Table]) -> "BoundBatches":
        """The C views of a list of batches, built once for repeated runs (an
        engine holds these as plain arrays; building them per call is host
        work that is not the runner's)."""
        keep: list = []
        nb = len(batches)
        views = (N.ColumnView * max(1, nb * self._ncols))()
        for b, table in enumerate(batches):
            arr, nc = _views(table, keep)
            if nc != self._ncols:
                raise ValueError("batch column count does not match the plan")
            for i in range(nc):
                views[b * nc + i] = arr[i]
        return BoundBatches(views, nb, keep)

    def run(self, batches, out: Optional[Sequence[N.Column]] = None, stream=None, raw: bool = False):
        """Runs every batch (a list of tables or the result of ``bind``);
        returns (columns per batch, rows per batch).  With ``raw`` the columns
        are returned as one C array of ``gx_column`` (free it with
        ``free_column_array``)."""
        bound = batches if isinstance(batches, BoundBatches) else self.bind(batches)
        nb = bound.count
        views = bound.views
        n = self.num_outputs
        outs = (N.Column * max(1, nb * n))()
        if out is not None:
            for i, c in enumerate(out):
                outs[i] = c
        rows = (C.c_int64 * max(1, nb))()
        s = _stream_handle(stream)
        st = N.StatusInfo()
        N.check(N.lib().gx_batch_runner_run(self._h, views, nb, self._ncols, outs, rows, s, C.byref(st)), st)
        if raw:
            return outs, list(rows[:nb])
        if out is not None:
            cols = [[outs[b * n + j] for j in range(n)] for b in range(nb)]
        else:
            cols = [[NativeColumn(N.Column(outs[b * n + j].type_id, 0, outs[b * n + j].data, outs[b * n + j].null_mask,
                                           outs[b * n + j].size, outs[b * n + j].capacity), s) for j in range(n)]
                    for b in range(nb)]
        return cols, [rows[b] for b in range(nb)]

    def config(self):
        bt, w = C.c_int32(0), C.c_int32(0)
        N.lib().gx_batch_runner_config(self._h, C.byref(bt), C.byref(w))
        return bt.value, w.value

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                N.lib().gx_batch_runner_destroy(self._h)
                self._h = None
        except Exception:
            pass


class BatchStream:
    """A persistent kernel of one filter plan fed batch by batch while it runs
    (gx_batch_stream_*): ``start`` launches it, ``push`` hands it a batch (the
    batch's columns must stay alive until ``finish``), ``finish`` closes the
    queue and returns (columns, rows) per pushed batch."""

    def __init__(self, plan: Plan, max_batches: int, max_total_rows: int, block_threads: int = 0,
                 words_per_warp: int = 0):
        st = N.StatusInfo()
        h = N.lib().gx_batch_stream_create(plan._h, max_batches, max_total_rows, block_threads, words_per_warp,
                                           C.byref(st))
        if not h:
            raise N.GxError(st.code, st.message.decode(errors="replace"))
        self._h = h
        self.num_outputs = plan.num_outputs
        self._ncols = len(plan.schema)
        self._keep: list = []
        self._count = 0
        self._stream = 0

    def start(self, stream=None) -> None:
        st = N.StatusInfo()
        self._stream = _stream_handle(stream)
        N.check(N.lib().gx_batch_stream_start(self._h, self._stream, C.byref(st)), st)
        self._keep, self._count = [], 0

    def push(self, table: Table) -> int:
        views, nc = _views(table, self._keep)
        self._keep.append(views)
        idx = C.c_int(-1)
        st = N.StatusInfo()
        N.check(N.lib().gx_batch_stream_push(self._h, views, nc, C.byref(idx), C.byref(st)), st)
        self._count += 1
        return idx.value

    def finish(self):
        n = self.num_outputs
        nb = self._count
        outs = (N.Column * max(1, nb * n))()
        rows = (C.c_int64 * max(1, nb))()
        st = N.StatusInfo()
        try:
            N.check(N.lib().gx_batch_stream_finish(self._h, outs, rows, nb, C.byref(st)), st)
        finally:
            self._keep, self._count = [], 0
        return [([NativeColumn(N.Column(outs[b * n + j].type_id, 0, outs[b * n + j].data, outs[b * n + j].null_mask,
                                        outs[b * n + j].size, outs[b * n + j].capacity), self._stream)
                  for j in range(n)], rows[b]) for b in range(nb)]

    def set_wait_polls(self, polls: int) -> None:
        """Test hook: polls (about 2 us apart) the kernel waits for a batch."""
        N.lib().gx_debug_batch_stream_wait_polls(self._h, polls)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                N.lib().gx_batch_stream_destroy(self._h)
                self._h = None
        except Exception:
            pass


class Learner:
    """Learned conjunct ordering over a stream of batches (gx_learner_*).

    Wraps a compiled filter ``Plan``; ``execute`` filters one batch and returns
    (columns, rows, info) where ``info`` is a dict of the batch report
    (path 0 = plain labelled batch, 1 = single pass; order, predicted and
    measured selectivities, re-runs, training loss)."""

    def __init__(self, plan: Plan, policy: int = N.GX_LEARN_POLICY_LEARNED, **options):
        L = N.lib()
        o = N.LearnerOptions()
        L.gx_learner_options_init(C.byref(o))
        o.policy = policy
        for k, v in options.items():
            if not hasattr(o, k):
                raise TypeError(f"unknown learner option {k!r}")
            setattr(o, k, v)
        st = N.StatusInfo()
        h = L.gx_learner_create(plan._h, C.byref(o), C.byref(st))
        if not h:
            raise N.GxError(st.code, st.message.decode(errors="replace"))
        self._h = h
        self.num_outputs = plan.num_outputs
        self.num_conjuncts = plan.num_conjuncts

    def execute(self, table: Table, stream=None):
        keep: list = []
        views, nc = _views(table, keep)
        s = _stream_handle(stream)
        n = self.num_outputs
        if not hasattr(self, "_outs"):
            self._outs = (N.Column * max(1, n))()
            self._rows = C.c_int64(0)
            self._st = N.StatusInfo()
        outs = self._outs
        for i in range(n):
            outs[i] = N.Column()
        info = N.LearnedBatchInfo()
        N.check(N.lib().gx_learner_execute(self._h, views, nc, outs, C.byref(self._rows), C.byref(info), s,
                                           C.byref(self._st)), self._st)
        return _wrap(outs, n, s), self._rows.value, _BatchReport(info)

    def execute_batches(self, tables: Sequence[Table], stream=None):
        """A queue of batches in one native call (gx_learner_execute_batches):
        each next batch is prepared while the current one runs.  Returns one
        (columns, rows, info) per batch."""
        q = self.queue_args(tables)
        self.run_queue(q, stream)
        return self.queue_results(q)

    def queue_args(self, tables: Sequence[Table]) -> "_Queue":
        """The native arguments of a batch queue, built once (run_queue runs it)."""
        keep: list = []
        nb = len(tables)
        arrs = [_views(t, keep) for t in tables]
        nc = arrs[0][1] if arrs else 0
        if any(k != nc for _, k in arrs):
            raise ValueError("every batch of a queue needs the same number of columns")
        ptrs = (C.POINTER(N.ColumnView) * max(1, nb))(*[C.cast(a, C.POINTER(N.ColumnView)) for a, _ in arrs])
        n = self.num_outputs
        return _Queue(keep=(keep, arrs), ptrs=ptrs, nc=nc, nb=nb, outs=(N.Column * max(1, nb * n))(),
                      rows=(C.c_int64 * max(1, nb))(), infos=(N.LearnedBatchInfo * max(1, nb))(), stream=0)

    def run_queue(self, q: "_Queue", stream=None) -> None:
        """The gx_learner_execute_batches call itself."""
        q.stream = _stream_handle(stream)
        st = N.StatusInfo()
        N.check(N.lib().gx_learner_execute_batches(self._h, q.ptrs, q.nc, q.nb, q.outs, q.rows, q.infos, q.stream,
                                                   C.byref(st)), st)

    def queue_results(self, q: "_Queue"):
        n = self.num_outputs
        res = []
        for b in range(q.nb):
            cols = [NativeColumn(N.Column(o.type_id, 0, o.data, o.null_mask, o.size, o.capacity), q.stream)
                    for o in q.outs[b * n:(b + 1) * n]]
            res.append((cols, q.rows[b], _BatchReport(q.infos[b])))
        return res

    def prepare(self, table: Table, stream=None) -> None:
        """Look-ahead: compute the prediction of a batch a later execute() gets."""
        keep: list = []
        views, nc = _views(table, keep)
        st = N.StatusInfo()
        N.check(N.lib().gx_learner_prepare(self._h, views, nc, _stream_handle(stream), C.byref(st)), st)

    def features(self, table: Table, stream=None):
        """The sketch features of one batch and the per-column anchors
        (gx_debug_learner_features)."""
        import numpy as np
        keep: list = []
        views, nc = _views(table, keep)
        f = np.zeros(32 * 11, dtype=np.float32)
        a = np.zeros(32, dtype=np.float64)
        k = C.c_int(0)
        st = N.StatusInfo()
        N.check(N.lib().gx_debug_learner_features(self._h, views, nc, f.ctypes.data_as(C.POINTER(C.c_float)),
                                                  f.size, C.byref(k), a.ctypes.data_as(C.POINTER(C.c_double)),
                                                  _stream_handle(stream), C.byref(st)), st)
        return f[:k.value], a[:k.value // 11]

    def save(self, path: str) -> None:
        st = N.StatusInfo()
        N.check(N.lib().gx_learner_save(self._h, path.encode(), C.byref(st)), st)

    def load(self, path: str) -> None:
        st = N.StatusInfo()
        N.check(N.lib().gx_learner_load(self._h, path.encode(), C.byref(st)), st)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                N.lib().gx_learner_destroy(self._h)
                self._h = None
        except Exception:
            pass


def mlp_grad(F: int, H: int, O: int, params, X, Y):
    """One forward + backward pass of the learner's MLP on the GPU
    (gx_debug_mlp_grad).  Returns (grad, loss, z) as numpy float32 arrays."""
    import numpy as np
    params = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    Y = np.ascontiguousarray(Y, dtype=np.float32)
    M = X.shape[0]
    grad = np.zeros_like(params)
    z = np.zeros((M, O), dtype=np.float32)
    loss = np.zeros(1, dtype=np.float32)
    fp = C.POINTER(C.c_float)
    st = N.StatusInfo()
    N.check(N.lib().gx_debug_mlp_grad(F, H, O, params.ctypes.data_as(fp), X.ctypes.data_as(fp), M,
                                      Y.ctypes.data_as(fp), grad.ctypes.data_as(fp), loss.ctypes.data_as(fp),
                                      z.ctypes.data_as(fp), C.byref(st)), st)
    return grad, float(loss[0]), z


def filter_aggregate(table: Table, condition: Optional[str], group_columns: Sequence[int],
                     aggregations: Sequence[Tuple[int, str]], stream=None) -> Tuple[List[NativeColumn], int]:
    """gx_filter_aggregate: the group-by aggregation of the rows passing
    ``condition``; ``aggregations`` holds (GX_AGG_* kind, input expression or
    "" for COUNT(*)).  Returns (keys then aggregation columns, groups); groups
    come in no particular order."""
    keep: list = []
    views, nc = _views(table, keep)
    s = _stream_handle(stream)
    nk, na = len(group_columns), len(aggregations)
    keys = (C.c_int * max(1, nk))(*group_columns)
    inputs = (C.c_char_p * max(1, na))(*[e.encode() for _, e in aggregations])
    kinds = (C.c_int * max(1, na))(*[k for k, _ in aggregations])
    outs = (N.Column * (nk + na))()
    groups = C.c_int64(0)
    st = N.StatusInfo()
    N.check(N.lib().gx_filter_aggregate(views, nc, condition.encode() if condition else None, keys, nk, inputs,
                                        kinds, na, outs, C.byref(groups), s, C.byref(st)), st)
    return _wrap(outs, nk + na, s), groups.value


def skip_data_rewrite(condition: str, dropped: Sequence[int] = (), prefix_form: bool = False) -> Tuple[str, bool]:
    """gx_skip_data_rewrite: the row-group statistics form of a condition
    (no GPU).  Returns (text, usable)."""
    d = (C.c_int * max(1, len(dropped)))(*dropped)
    buf = C.create_string_buffer(8192)
    usable = C.c_int(0)
    st = N.StatusInfo()
    N.check(N.lib().gx_skip_data_rewrite(condition.encode(), d, len(dropped), 1 if prefix_form else 0, buf,
                                         len(buf), C.byref(usable), C.byref(st)), st)
    return buf.value.decode(), bool(usable.value)


def skip_data_filter(metadata: Table, metadata_names: Sequence[str], column_names: Sequence[str],
                     table_scan: str, stream=None):
    """gx_skip_data_filter: the (file, row group) ids a TableScan's condition
    cannot rule out, from the row-group statistics table.  Returns
    (columns, rows), or (None, 0) when the condition allows no pruning."""
    keep: list = []
    views, nc = _views(metadata, keep)
    mnames = (C.c_char_p * max(1, nc))(*[x.encode() for x in metadata_names])
    cnames = (C.c_char_p * max(1, len(column_names)))(*[x.encode() for x in column_names])
    outs = (N.Column * 2)()
    rows = C.c_int64(0)
    unusable = C.c_int(0)
    s = _stream_handle(stream)
    st = N.StatusInfo()
    N.check(N.lib().gx_skip_data_filter(views, mnames, nc, cnames, len(column_names), table_scan.encode(), outs,
                                        C.byref(rows), C.byref(unusable), s, C.byref(st)), st)
    if unusable.value:
        return None, 0
    return _wrap(outs, 2, s), rows.value


def aggregate_check(schema: Sequence[int], has_mask: Sequence[bool], condition: Optional[str],
                    group_columns: Sequence[int], aggregations: Sequence[Tuple[int, str]]):
    """gx_debug_aggregate_check: builds and NVRTC-compiles the aggregation
    kernel (no GPU needed); returns (registers, spill bytes, shared bytes)."""
    nc, nk, na = len(schema), len(group_columns), len(aggregations)
    types = (C.c_int32 * max(1, nc))(*[int(t) for t in schema])
    masks = (C.c_uint8 * max(1, nc))(*[1 if m else 0 for m in has_mask])
    keys = (C.c_int * max(1, nk))(*group_columns)
    inputs = (C.c_char_p * max(1, na))(*[e.encode() for _, e in aggregations])
    kinds = (C.c_int * max(1, na))(*[k for k, _ in aggregations])
    r, sp, sh = C.c_int32(0), C.c_int32(0), C.c_int32(0)
    st = N.StatusInfo()
    N.check(N.lib().gx_debug_aggregate_check(types, masks, nc, condition.encode() if condition else None, keys, nk,
                                             inputs, kinds, na, C.byref(r), C.byref(sp), C.byref(sh),
                                             C.byref(st)), st)
    return r.value, sp.value, sh.value


def free_columns(cols: Sequence[NativeColumn], stream=None) -> None:
    """Releases library-owned output columns with one gx_free_columns call."""
    live = [c for c in cols if c._c.data]
    if not live:
        return
    arr = (N.Column * len(live))(*[c._c for c in live])
    N.lib().gx_free_columns(arr, len(live), _stream_handle(stream) if stream is not None else live[0]._stream)
    for c in live:
        c._c.data = None
        c._c.null_mask = None


def set_current_timestamp(timestamp: Optional[str]) -> None:
    """The calling thread's query timestamp for CURRENT_DATE / CURRENT_TIMESTAMP
    ("YYYY-MM-DD hh:mm:ss[.fraction]"; None clears it)."""
    st = N.StatusInfo()
    N.check(N.lib().gx_set_current_timestamp(timestamp.encode() if timestamp else None, C.byref(st)), st)


def preprocess(expression: str, schema: Sequence[int] = (), stages: int = 31) -> str:
    """preprocess_expression's text rewrites (gx_debug_preprocess_expression)."""
    st = N.StatusInfo()
    buf = C.create_string_buffer(8192)
    types = (C.c_int32 * max(1, len(schema)))(*[int(t) for t in schema])
    N.check(N.lib().gx_debug_preprocess_expression(expression.encode(), types, len(schema), stages, buf, 8192,
                                                   C.byref(st)), st)
    return buf.value.decode()


def version() -> str:
    return N.lib().gx_version().decode()


def jit_stats():
    c = C.c_int64(0)
    ms = C.c_double(0)
    N.lib().gx_debug_jit_stats(C.byref(c), C.byref(ms))
    return c.value, ms.value


def fail_next_allocation(n: int = 1) -> None:
    """Host-side fault injection: the n-th next device allocation fails (GX_ERR_OOM)."""
    N.lib().gx_debug_fail_allocation(n)
