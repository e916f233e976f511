"""CPU oracle of the fused filter + group-by aggregation (test infrastructure).

Restates the aggregation step of BlazingSQL's Filter -> Projection ->
Aggregate chain, engine/src/operators/GroupBy.cpp:
  - compute_aggregations_with_groupby (:316-416): aggregation inputs are the
    columns or the evaluate_expressions results of their expressions
    (:346-353), grouped by the key columns with NULL keys as a group of their
    own (cudf::null_policy::INCLUDE, :380); output = keys, then aggregations
    in request order (:383-405); SUM0 of a group without valid input is 0
    (:394-397);
  - compute_aggregations_without_groupby (:217-314): one output row, empty
    input included; COUNT(*) = rows (:228-232), COUNT(x) = valid inputs
    (:253-257);
  - output types (:30-57): COUNT INT64; SUM widened to INT64 / FLOAT64;
    MIN / MAX the input's type; MEAN FLOAT64.
SUM / MIN / MAX / MEAN of a group without valid input are NULL (cudf's
aggregation result for an all-null group).  Integer sums wrap (two's
complement); floating sums add sequentially in row order.

The filter and the aggregation-input expressions go through the C++ oracle
(oracle/gx_oracle.cpp), so the row semantics are the ones pinned there.
Groups come out ordered by key, NULL before any value (the device returns
them unordered; tests sort them the same way).  Only tests/ and bench.py's
CPU-baseline leg use this module.
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np

from blazingsql_gb300.types import HostColumn, TypeId as T, is_float, np_dtype, pack_validity, unpack_validity
from oracle import pyoracle

SUM, SUM0, MIN, MAX, COUNT_VALID, COUNT_ALL, MEAN = range(7)


def _wrap64(v: int) -> int:
    v &= (1 << 64) - 1
    return v - (1 << 64) if v >= (1 << 63) else v


def output_types(schema: Sequence[int], group_columns: Sequence[int], kinds: Sequence[int],
                 input_types: Sequence[Optional[int]]) -> List[int]:
    out = [schema[c] for c in group_columns]
    for k, t in zip(kinds, input_types):
        if k in (COUNT_VALID, COUNT_ALL):
            out.append(T.INT64)
        elif k == MEAN:
            out.append(T.FLOAT64)
        elif k in (SUM, SUM0):
            out.append(T.FLOAT64 if is_float(t) else T.INT64)
        else:
            out.append(t)
    return out


def filter_aggregate(cols: Sequence[HostColumn], condition: Optional[str], group_columns: Sequence[int],
                     aggregations: Sequence[Tuple[int, str]], nthreads: int = 4) -> List[HostColumn]:
    schema = [c.type_id for c in cols]
    exprs = [f"${c}" for c in group_columns] + [e for k, e in aggregations if k != COUNT_ALL]
    if condition:
        ev, rows = pyoracle.filter_project(cols, condition, exprs, nthreads)
    else:
        ev = pyoracle.evaluate_expressions(cols, exprs, nthreads)
        rows = cols[0].data.shape[0] if cols else 0
    nk = len(group_columns)
    vals = [np.asarray(c.data[:rows]) for c in ev]
    valid = [unpack_validity(c.mask, rows) for c in ev]
    # aggregation i -> evaluated column index (None for COUNT(*))
    src: List[Optional[int]] = []
    nxt = nk
    for k, _ in aggregations:
        if k == COUNT_ALL:
            src.append(None)
        else:
            src.append(nxt)
            nxt += 1
    in_types = [None if s is None else ev[s].type_id for s in src]
    # groups in row order of first appearance
    groups = {}
    for r in range(rows):
        key = tuple(int(vals[j][r]) if valid[j][r] else None for j in range(nk))
        groups.setdefault(key, []).append(r)
    if nk == 0 and not groups:
        groups[()] = []
    keys = sorted(groups, key=lambda kt: tuple((0, 0) if v is None else (1, v) for v in kt))
    out_types = output_types(schema, group_columns, [k for k, _ in aggregations], in_types)
    G = len(keys)
    data = [np.zeros(G, dtype=np_dtype(t)) for t in out_types]
    ok = [np.zeros(G, dtype=bool) for _ in out_types]
    for gi, key in enumerate(keys):
        idx = groups[key]
        for j in range(nk):
            ok[j][gi] = key[j] is not None
            data[j][gi] = 0 if key[j] is None else key[j]
        for i, (k, _) in enumerate(aggregations):
            o = nk + i
            if k == COUNT_ALL:
                data[o][gi] = len(idx)
                ok[o][gi] = True
                continue
            s = src[i]
            vv = [vals[s][r] for r in idx if valid[s][r]]
            flt = is_float(in_types[i])
            if k == COUNT_VALID:
                data[o][gi] = len(vv)
                ok[o][gi] = True
            elif k in (SUM, SUM0, MEAN):
                if flt:
                    acc = 0.0
                    for v in vv:
                        acc = float(np.float64(acc) + np.float64(v))
                else:
                    acc = _wrap64(sum(int(v) for v in vv))
                if k == MEAN:
                    if vv:
                        data[o][gi] = (acc if flt else float(acc)) / float(len(vv))
                        ok[o][gi] = True
                else:
                    if vv or k == SUM0:
                        data[o][gi] = acc
                        ok[o][gi] = True
            else:  # MIN / MAX
                if vv:
                    data[o][gi] = min(vv) if k == MIN else max(vv)
                    ok[o][gi] = True
    return [HostColumn(t, d, pack_validity(v)) for t, d, v in zip(out_types, data, ok)]
