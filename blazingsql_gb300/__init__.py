"""GB300-native row-wise expression evaluator (filter + project) for BlazingSQL plans.

The product is the native library ``_lib/libgxeval.so`` (C ABI in
``include/gx_eval.h``); this package is a thin host mirror over it.
"""
from .types import HostColumn, TypeId, pack_validity, unpack_validity  # noqa: F401
from ._native import (GxError, GX_LEARN_POLICY_LEARNED, GX_LEARN_POLICY_PLAIN,  # noqa: F401
                      GX_LEARN_POLICY_TEXTUAL, GX_AGG_SUM, GX_AGG_SUM0, GX_AGG_MIN, GX_AGG_MAX,
                      GX_AGG_COUNT_VALID, GX_AGG_COUNT_ALL, GX_AGG_MEAN)
from .api import (BatchRunner, BatchStream, DeviceColumn, Learner, NativeColumn, Plan, evaluate_expressions, filter_project,  # noqa: F401
                  filter_aggregate, process_filter, process_project, version)
from . import api  # noqa: F401
