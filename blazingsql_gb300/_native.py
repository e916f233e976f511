"""ctypes binding of the C ABI in include/gx_eval.h (libgxeval.so).

The library is built in-tree by ``blazingsql_gb300.build_ext.build()``.  There
is no CPU fallback: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgxeval.so")

GX_OK = 0
GX_ERR_PARSE = 1
GX_ERR_UNSUPPORTED = 2
GX_ERR_TYPE = 3
GX_ERR_OOM = 4
GX_ERR_CUDA = 5
GX_ERR_TIMEOUT = 6
GX_ERR_INVALID = 7
GX_ERR_CAPACITY = 8

# gx_plan_execute_noalloc: tile status words of its fixed scratch array, and the
# largest batch that fits with the default 512-row tile (4 warps x 4 words x 32)
GX_NOALLOC_MAX_TILES = 524284
GX_NOALLOC_MAX_ROWS = GX_NOALLOC_MAX_TILES * 512

GX_AGG_SUM, GX_AGG_SUM0, GX_AGG_MIN, GX_AGG_MAX, GX_AGG_COUNT_VALID, GX_AGG_COUNT_ALL, GX_AGG_MEAN = range(7)
GX_FILTER_AUTO = 0
GX_FILTER_TWO_PASS = 1
GX_FILTER_SINGLE_PASS = 2


class GxError(RuntimeError):
    """A non-OK status from the evaluator; ``code`` is the gx_status value."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[gx status {code}] {message}")
        self.code = code
        self.message = message

    @property
    def retryable(self) -> bool:
        return self.code == GX_ERR_OOM


class ColumnView(C.Structure):
    _fields_ = [("type_id", C.c_int32), ("reserved", C.c_int32), ("data", C.c_void_p),
                ("null_mask", C.c_void_p), ("offset", C.c_int64), ("size", C.c_int64),
                ("string_offsets", C.c_void_p)]


class Column(C.Structure):
    _fields_ = [("type_id", C.c_int32), ("reserved", C.c_int32), ("data", C.c_void_p),
                ("null_mask", C.c_void_p), ("size", C.c_int64), ("capacity", C.c_int64),
                ("string_offsets", C.c_void_p), ("string_bytes", C.c_int64)]


class StatusInfo(C.Structure):
    _fields_ = [("code", C.c_int32), ("message", C.c_char * 500)]


class PlanOptions(C.Structure):
    _fields_ = [("filter_mode", C.c_int32), ("block_threads", C.c_int32), ("words_per_warp", C.c_int32),
                ("use_tma", C.c_int32), ("short_circuit", C.c_int32), ("num_conjuncts", C.c_int32),
                ("conjunct_order", C.c_int32 * 16), ("rand_seed", C.c_uint64)]


class LearnerOptions(C.Structure):
    _fields_ = [("policy", C.c_int32), ("warmup_batches", C.c_int32), ("relabel_every", C.c_int32),
                ("train_steps", C.c_int32), ("learning_rate", C.c_float), ("hidden", C.c_int32),
                ("capacity_margin", C.c_double), ("capacity_slack", C.c_int64), ("sketch_stride_words", C.c_int64),
                ("async_training", C.c_int32), ("fast_words_per_warp", C.c_int32), ("seed", C.c_uint64),
                ("size_outputs", C.c_int32), ("reserved", C.c_int32)]


class LearnedBatchInfo(C.Structure):
    _fields_ = [("path", C.c_int32), ("reruns", C.c_int32), ("rows", C.c_int64), ("predicted_rows", C.c_int64),
                ("train_loss", C.c_float), ("num_conjuncts", C.c_int32), ("order", C.c_int32 * 16),
                ("predicted_sel", C.c_double * 16), ("measured_sel", C.c_double * 16)]


GX_LEARN_POLICY_LEARNED, GX_LEARN_POLICY_PLAIN, GX_LEARN_POLICY_TEXTUAL = 0, 1, 2

_lib = None


def lib():
    """Loads libgxeval.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"native evaluator library missing ({LIB_PATH}); build it with "
                           "blazingsql_gb300.build_ext.build() -- there is no CPU fallback")
    L = C.CDLL(LIB_PATH)
    P = C.POINTER
    L.gx_version.restype = C.c_char_p
    L.gx_evaluate_expressions.argtypes = [P(ColumnView), C.c_int, P(C.c_char_p), C.c_int, P(Column), C.c_void_p,
                                          P(StatusInfo)]
    L.gx_process_project.argtypes = [P(ColumnView), C.c_int, C.c_char_p, P(Column), C.c_int, P(C.c_int),
                                     C.c_char_p, C.c_int, C.c_void_p, P(StatusInfo)]
    L.gx_process_filter.argtypes = [P(ColumnView), C.c_int, C.c_char_p, P(Column), P(C.c_int64), C.c_void_p,
                                    P(StatusInfo)]
    L.gx_filter_project.argtypes = [P(ColumnView), C.c_int, C.c_char_p, P(C.c_char_p), C.c_int, P(Column),
                                    P(C.c_int64), C.c_void_p, P(StatusInfo)]
    L.gx_free_columns.argtypes = [P(Column), C.c_int, C.c_void_p]
    L.gx_free_columns.restype = None
    L.gx_column_to_host.argtypes = [P(Column), C.c_void_p, C.c_void_p, C.c_void_p, P(StatusInfo)]
    L.gx_string_offsets_to_host.argtypes = [P(Column), C.c_void_p, C.c_void_p, P(StatusInfo)]
    L.gx_debug_like_automaton.argtypes = [C.c_char_p, C.c_char_p, C.c_int64, P(C.c_int32), P(StatusInfo)]
    L.gx_plan_options_init.argtypes = [P(PlanOptions)]
    L.gx_plan_options_init.restype = None
    L.gx_plan_compile.argtypes = [P(C.c_int32), P(C.c_uint8), C.c_int, C.c_char_p, P(C.c_char_p), C.c_int,
                                  P(PlanOptions), P(StatusInfo)]
    L.gx_plan_compile.restype = C.c_void_p
    L.gx_plan_num_outputs.argtypes = [C.c_void_p]
    L.gx_plan_output_type.argtypes = [C.c_void_p, C.c_int]
    L.gx_plan_output_type.restype = C.c_int32
    L.gx_plan_num_conjuncts.argtypes = [C.c_void_p]
    L.gx_plan_execute.argtypes = [C.c_void_p, P(ColumnView), C.c_int, P(Column), P(C.c_int64), C.c_void_p,
                                  P(StatusInfo)]
    L.gx_plan_execute_noalloc.argtypes = [C.c_void_p, P(ColumnView), C.c_int, P(Column), P(C.c_int64), C.c_void_p,
                                          P(StatusInfo)]
    L.gx_plan_destroy.argtypes = [C.c_void_p]
    L.gx_plan_destroy.restype = None
    L.gx_debug_kernel_source.argtypes = [C.c_void_p, C.c_int, P(C.c_uint8), C.c_char_p, C.c_int64, P(StatusInfo)]
    L.gx_debug_kernel_source.restype = C.c_int64
    L.gx_debug_compile_check.argtypes = [C.c_void_p, C.c_int, P(C.c_uint8), P(StatusInfo)]
    L.gx_batch_runner_create.argtypes = [C.c_void_p, C.c_int, C.c_int64, C.c_int, P(StatusInfo)]
    L.gx_batch_runner_create.restype = C.c_void_p
    L.gx_batch_runner_run.argtypes = [C.c_void_p, P(ColumnView), C.c_int, C.c_int, P(Column), P(C.c_int64),
                                      C.c_void_p, P(StatusInfo)]
    L.gx_batch_runner_config.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32)]
    L.gx_batch_runner_destroy.argtypes = [C.c_void_p]
    L.gx_batch_runner_destroy.restype = None
    L.gx_batch_stream_create.argtypes = [C.c_void_p, C.c_int, C.c_int64, C.c_int, C.c_int, P(StatusInfo)]
    L.gx_batch_stream_create.restype = C.c_void_p
    L.gx_batch_stream_start.argtypes = [C.c_void_p, C.c_void_p, P(StatusInfo)]
    L.gx_batch_stream_push.argtypes = [C.c_void_p, P(ColumnView), C.c_int, P(C.c_int), P(StatusInfo)]
    L.gx_batch_stream_finish.argtypes = [C.c_void_p, P(Column), P(C.c_int64), C.c_int, P(StatusInfo)]
    L.gx_batch_stream_destroy.argtypes = [C.c_void_p]
    L.gx_batch_stream_destroy.restype = None
    L.gx_debug_batch_stream_wait_polls.argtypes = [C.c_void_p, C.c_uint32]
    L.gx_debug_kernel_resources.argtypes = [C.c_void_p, C.c_int, P(C.c_uint8), P(C.c_int32), P(C.c_int32),
                                            P(C.c_int32), P(StatusInfo)]
    L.gx_debug_fail_allocation.argtypes = [C.c_int]
    L.gx_debug_fail_allocation.restype = None
    L.gx_set_current_timestamp.argtypes = [C.c_char_p, P(StatusInfo)]
    L.gx_debug_preprocess_expression.argtypes = [C.c_char_p, P(C.c_int32), C.c_int, C.c_int, C.c_char_p, C.c_int,
                                                 P(StatusInfo)]
    L.gx_debug_filter_timeout.argtypes = [C.c_void_p, P(ColumnView), C.c_int, C.c_int64, C.c_uint32, P(StatusInfo)]
    L.gx_debug_jit_stats.argtypes = [P(C.c_int64), P(C.c_double)]
    L.gx_debug_jit_stats.restype = None
    L.gx_debug_rebuild_expression.argtypes = [C.c_char_p, C.c_char_p, C.c_int, P(StatusInfo)]
    L.gx_debug_set_kernel_timing.argtypes = [C.c_int]
    L.gx_debug_set_kernel_timing.restype = None
    L.gx_debug_kernel_ms.argtypes = [C.c_int]
    L.gx_debug_kernel_ms.restype = C.c_double
    L.gx_debug_launch_count.argtypes = []
    L.gx_debug_launch_count.restype = C.c_int64
    L.gx_learner_options_init.argtypes = [P(LearnerOptions)]
    L.gx_learner_options_init.restype = None
    L.gx_learner_create.argtypes = [C.c_void_p, P(LearnerOptions), P(StatusInfo)]
    L.gx_learner_create.restype = C.c_void_p
    L.gx_learner_execute.argtypes = [C.c_void_p, P(ColumnView), C.c_int, P(Column), P(C.c_int64),
                                     P(LearnedBatchInfo), C.c_void_p, P(StatusInfo)]
    L.gx_filter_aggregate.argtypes = [P(ColumnView), C.c_int, C.c_char_p, P(C.c_int), C.c_int, P(C.c_char_p),
                                      P(C.c_int), C.c_int, P(Column), P(C.c_int64), C.c_void_p, P(StatusInfo)]
    L.gx_debug_aggregate_check.argtypes = [P(C.c_int32), P(C.c_uint8), C.c_int, C.c_char_p, P(C.c_int), C.c_int,
                                           P(C.c_char_p), P(C.c_int), C.c_int, P(C.c_int32), P(C.c_int32),
                                           P(C.c_int32), P(StatusInfo)]
    L.gx_skip_data_rewrite.argtypes = [C.c_char_p, P(C.c_int), C.c_int, C.c_int, C.c_char_p, C.c_int, P(C.c_int),
                                       P(StatusInfo)]
    L.gx_skip_data_filter.argtypes = [P(ColumnView), P(C.c_char_p), C.c_int, P(C.c_char_p), C.c_int, C.c_char_p,
                                      P(Column), P(C.c_int64), P(C.c_int), C.c_void_p, P(StatusInfo)]
    L.gx_plan_execute_host.argtypes = [C.c_void_p, P(ColumnView), C.c_int, P(Column), P(C.c_int64), C.c_void_p,
                                       P(StatusInfo)]
    L.gx_learner_prepare.argtypes = [C.c_void_p, P(ColumnView), C.c_int, C.c_void_p, P(StatusInfo)]
    L.gx_learner_execute_batches.argtypes = [C.c_void_p, P(P(ColumnView)), C.c_int, C.c_int, P(Column),
                                             P(C.c_int64), P(LearnedBatchInfo), C.c_void_p, P(StatusInfo)]
    L.gx_learner_save.argtypes = [C.c_void_p, C.c_char_p, P(StatusInfo)]
    L.gx_learner_load.argtypes = [C.c_void_p, C.c_char_p, P(StatusInfo)]
    L.gx_learner_destroy.argtypes = [C.c_void_p]
    L.gx_learner_destroy.restype = None
    fp = P(C.c_float)
    L.gx_debug_learner_features.argtypes = [C.c_void_p, P(ColumnView), C.c_int, fp, C.c_int, P(C.c_int),
                                            P(C.c_double), C.c_void_p, P(StatusInfo)]
    L.gx_debug_mlp_grad.argtypes = [C.c_int, C.c_int, C.c_int, fp, fp, C.c_int, fp, fp, fp, fp, P(StatusInfo)]
    _lib = L
    return L


def check(rc: int, st: StatusInfo) -> None:
    if rc != GX_OK:
        raise GxError(rc, st.message.decode(errors="replace"))


# every symbol declared in include/gx_eval.h
EXPORTED_SYMBOLS = [
    "gx_evaluate_expressions", "gx_process_project", "gx_process_filter", "gx_filter_project", "gx_free_columns",
    "gx_column_to_host", "gx_string_offsets_to_host", "gx_debug_like_automaton", "gx_plan_options_init", "gx_plan_compile", "gx_plan_num_outputs", "gx_plan_output_type",
    "gx_plan_num_conjuncts", "gx_plan_execute", "gx_plan_execute_noalloc", "gx_plan_destroy", "gx_version",
    "gx_debug_kernel_source",
    "gx_debug_compile_check", "gx_debug_fail_allocation", "gx_debug_filter_timeout", "gx_set_current_timestamp",
    "gx_debug_preprocess_expression", "gx_debug_jit_stats", "gx_debug_rebuild_expression",
    "gx_debug_set_kernel_timing", "gx_debug_kernel_ms", "gx_debug_launch_count",
    "gx_learner_options_init", "gx_learner_create", "gx_learner_execute", "gx_learner_prepare", "gx_learner_save",
    "gx_learner_execute_batches", "gx_plan_execute_host", "gx_filter_aggregate", "gx_debug_aggregate_check",
    "gx_skip_data_rewrite", "gx_skip_data_filter",
    "gx_learner_load",
    "gx_learner_destroy", "gx_debug_mlp_grad", "gx_debug_learner_features", "gx_debug_kernel_resources",
    "gx_batch_runner_create", "gx_batch_runner_run", "gx_batch_runner_config", "gx_batch_runner_destroy",
    "gx_batch_stream_create", "gx_batch_stream_start", "gx_batch_stream_push", "gx_batch_stream_finish",
    "gx_batch_stream_destroy", "gx_debug_batch_stream_wait_polls",
]


def rebuild_expression(expr: str) -> str:
    """The product parser's lowered form of one expression, as text."""
    buf = C.create_string_buffer(8192)
    st = StatusInfo()
    check(lib().gx_debug_rebuild_expression(expr.encode(), buf, 8192, C.byref(st)), st)
    return buf.value.decode()
