"""Synthetic workloads with the shapes, sizes and value distributions of the
evaluator's benchmark configurations, plus their frozen plans.

C1 plain       2^24 rows: INT64 U[0,1e6), FLOAT64 N(0,1), INT32 U[-1000,1000] with 10% nulls
C2 deep        2^28 rows: 2x INT64 U[0,2^40), 2x FLOAT64 N(0,1e3), DATE days over 2557 days
               from 1992-01-01, INT8 U{0..5}; 5% nulls each; frozen 12-level plan
C3 batched     C2's plan over 512 batches, sizes log-uniform in [1K, 4M]
C4 learned     8 Zipf(1.2) INT64/FLOAT64 columns, 6 AND-ed range/equality conjuncts
C5 order-line  600M rows (quantity, price, discount, tax, shipdate, two flags), 4M-row batches

Generation runs on the device (torch, seeded) so large inputs never cross PCIe/C2C;
``host=True`` variants return numpy (HostColumn) for the CPU oracle.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from .types import HostColumn, TypeId as T, np_dtype, pack_validity

DAY_1992_01_01 = 8035          # days since 1970-01-01
DAYS_7Y = 2557                 # 1992-01-01 .. 1998-12-31

# ---------------------------------------------------------------- frozen plans
C1_CONDITION = "AND(>($0, 500000), <($1, 0.5))"
C1_PROJECTIONS = ["+(*($0, 3), $2)", "/($1, CAST($2):DOUBLE)"]

# 12 levels deep as RexNode text (CASE > + > * > FLOOR > / > CASE > - > CAST > MOD > ABS > - > $1),
# using CASE, COALESCE (Calcite's CASE(IS NOT NULL(a), a, b) form), IS NULL, MOD, FLOOR,
# casts, LN and EXP on the float columns.
C2_CONDITION = "AND(IS NOT NULL($2), <=($4, 1996-12-31))"
C2_PROJECTIONS = [
    "CASE(IS NULL($5), FLOOR(LN(+(ABS($2), 1.0))), =($5, 0), EXP(/($3, 1000.0)), "
    "+(CAST(MOD(CASE(IS NOT NULL($0), $0, $1), 997)):DOUBLE, "
    "*(FLOOR(/(CASE(IS NOT NULL($3), -($3, CAST(MOD(ABS(-($1, $0)), 1000)):DOUBLE), $2), 10.0)), "
    "CAST($5):DOUBLE)))",
    "MOD(CASE(IS NOT NULL($0), $0, $1), 997)",
]

# TPC-H Q1's aggregation shape over the order-line columns (C5), grouped by
# the two flag columns: (gx_agg_kind, input expression); kinds 0 SUM, 2 MIN,
# 3 MAX, 5 COUNT(*), 6 MEAN.  Inputs are the quantity, price, charge
# (price x (100 - discount) x (100 + tax), exact INT64), unit price,
# discount fraction and ship date.
C5_AGG_KEYS = [5, 6]
C5_AGGREGATIONS = [(0, "$0"), (0, "$1"), (0, "*(*($1, -(100, $2)), +(100, $3))"),
                   (0, "/(CAST($1):DOUBLE, CAST($0):DOUBLE)"), (6, "$0"), (6, "/(CAST($2):DOUBLE, 100.0)"),
                   (5, ""), (2, "$4"), (3, "/(CAST($1):DOUBLE, CAST($0):DOUBLE)")]

# Six side-effect-free AND-ed range / equality conjuncts over Zipf(1.2) columns
# whose support is shifted per batch, so each conjunct's selectivity moves from
# about 0.1% to about 90% between batches ($3 and $7 are carried, not tested).
C4_CONDITION = "AND(>($0, 100000), =($1, 1000), <($2, 1000), <($4, 1000.0), >($5, 5000.0), <($6, 100.0))"
C4_PROJECTIONS = [f"${i}" for i in range(8)]
C4_ZIPF_S = 1.2
C4_ZIPF_MAX_RANK = 1_000_000
C4_BATCH_ROWS = 1 << 22

C5_CUTOFF = "1998-09-02"
C5_CONDITION = "<=($4, 1998-09-02)"
C5_PROJECTIONS = [
    "*(*($1, -(100, $2)), +(100, $3))",
    "/(CAST($1):DOUBLE, CAST($0):DOUBLE)",
    "/(CAST($2):DOUBLE, 100.0)",
    "$5",
    "$6",
]


@dataclass
class Workload:
    name: str
    schema: List[int]
    nullable: List[bool]
    condition: Optional[str]
    projections: List[str]
    rows: int
    # bytes per input row (referenced columns, values + validity bits)
    in_bytes_per_row: float = 0.0
    out_bytes_per_row: float = 0.0   # per surviving row
    notes: dict = field(default_factory=dict)

    def algorithmic_bytes(self, rows: int, out_rows: int) -> float:
        """N * sum_in(w + nullable/8) + N*s * sum_out(w + 1/8)."""
        return rows * self.in_bytes_per_row + out_rows * self.out_bytes_per_row


def _sizes(types: Sequence[int]) -> List[int]:
    return [np_dtype(t).itemsize for t in types]


def workload(name: str, rows: Optional[int] = None) -> Workload:
    if name == "c1":
        schema = [T.INT64, T.FLOAT64, T.INT32]
        nullable = [False, False, True]
        w = Workload("c1_plain_filter_project", schema, nullable, C1_CONDITION, list(C1_PROJECTIONS),
                     rows or (1 << 24))
        w.in_bytes_per_row = 8 + 8 + 4 + 1 / 8
        w.out_bytes_per_row = 8 + 8 + 2 / 8
        return w
    if name == "c2":
        schema = [T.INT64, T.INT64, T.FLOAT64, T.FLOAT64, T.TIMESTAMP_DAYS, T.INT8]
        w = Workload("c2_deep_filter_project", schema, [True] * 6, C2_CONDITION, list(C2_PROJECTIONS),
                     rows or (1 << 28))
        w.in_bytes_per_row = sum(_sizes(schema)) + 6 / 8
        w.out_bytes_per_row = 8 + 8 + 2 / 8
        return w
    if name == "c4":
        schema = [T.INT64] * 4 + [T.FLOAT64] * 4
        w = Workload("c4_learned_order_filter", schema, [False] * 8, C4_CONDITION, list(C4_PROJECTIONS),
                     rows or (1 << 28))
        w.in_bytes_per_row = 64.0
        w.out_bytes_per_row = 64 + 8 / 8
        w.notes = {"batch_rows": C4_BATCH_ROWS, "zipf_s": C4_ZIPF_S}
        return w
    if name == "c5":
        schema = [T.INT32, T.INT64, T.INT64, T.INT64, T.TIMESTAMP_DAYS, T.INT8, T.INT8]
        w = Workload("c5_orderline_filter_project", schema, [False] * 7, C5_CONDITION, list(C5_PROJECTIONS),
                     rows or 600_000_000)
        w.in_bytes_per_row = sum(_sizes(schema))
        w.out_bytes_per_row = 8 + 8 + 8 + 1 + 1 + 5 / 8
        return w
    raise ValueError(f"unknown workload {name}")


# ---------------------------------------------------------------- generators
def _np_columns(name: str, n: int, seed: int) -> List[HostColumn]:
    rng = np.random.default_rng(seed)
    if name == "c1":
        c0 = rng.integers(0, 1_000_000, n, dtype=np.int64)
        c1 = rng.normal(0.0, 1.0, n)
        c2 = rng.integers(-1000, 1001, n, dtype=np.int64).astype(np.int32)
        v2 = rng.random(n) >= 0.10
        return [HostColumn(T.INT64, c0), HostColumn(T.FLOAT64, c1), HostColumn(T.INT32, c2, pack_validity(v2))]
    if name == "c2":
        c0 = rng.integers(0, 1 << 40, n, dtype=np.int64)
        c1 = rng.integers(0, 1 << 40, n, dtype=np.int64)
        c2 = rng.normal(0.0, 1e3, n)
        c3 = rng.normal(0.0, 1e3, n)
        c4 = (DAY_1992_01_01 + rng.integers(0, DAYS_7Y, n)).astype(np.int32)
        c5 = rng.integers(0, 6, n).astype(np.int8)
        cols = [HostColumn(T.INT64, c0), HostColumn(T.INT64, c1), HostColumn(T.FLOAT64, c2),
                HostColumn(T.FLOAT64, c3), HostColumn(T.TIMESTAMP_DAYS, c4), HostColumn(T.INT8, c5)]
        for c in cols:
            c.mask = pack_validity(rng.random(n) >= 0.05)
        return cols
    if name == "c5":
        q = rng.integers(1, 51, n).astype(np.int32)
        price = rng.integers(90000, 10500001, n, dtype=np.int64)
        disc = rng.integers(0, 11, n, dtype=np.int64)
        tax = rng.integers(0, 9, n, dtype=np.int64)
        ship = (DAY_1992_01_01 + rng.integers(0, DAYS_7Y, n)).astype(np.int32)
        f1 = rng.integers(0, 3, n).astype(np.int8)
        f2 = rng.integers(0, 2, n).astype(np.int8)
        return [HostColumn(T.INT32, q), HostColumn(T.INT64, price), HostColumn(T.INT64, disc),
                HostColumn(T.INT64, tax), HostColumn(T.TIMESTAMP_DAYS, ship), HostColumn(T.INT8, f1),
                HostColumn(T.INT8, f2)]
    raise ValueError(name)


def c3_batch_sizes(seed: int = 3, nbatches: int = 512, lo: int = 1024, hi: int = 4194304) -> List[int]:
    """Execution-graph batch sizes: floor(exp(U[ln lo, ln hi])) per batch."""
    rng = np.random.default_rng(seed)
    return [int(np.exp(x)) for x in rng.uniform(np.log(lo), np.log(hi), nbatches)]


def slice_batches(cols, sizes: Sequence[int]):
    """Consecutive row ranges of one table as batches (views with offsets)."""
    from .api import DeviceColumn
    out = []
    start = 0
    for n in sizes:
        out.append([DeviceColumn(c.type_id, c.data, c.mask, c.offset + start, n, c.str_offsets) for c in cols])
        start += n
    return out


_ZIPF_CDF = None


def _zipf_cdf() -> np.ndarray:
    global _ZIPF_CDF
    if _ZIPF_CDF is None:
        p = np.arange(1, C4_ZIPF_MAX_RANK + 1, dtype=np.float64) ** -C4_ZIPF_S
        c = np.cumsum(p)
        _ZIPF_CDF = c / c[-1]
    return _ZIPF_CDF


def c4_shifts(seed: int, batch: int) -> List[float]:
    """Per-batch support shifts of the 8 C4 columns (value = shift + Zipf rank
    [+ U[0,1) for the FLOAT64 columns]).  Each shift puts its conjunct's
    boundary at a log-uniform rank, so the conjunct's selectivity varies per
    batch; the carried columns $3 and $7 get arbitrary shifts."""
    r = np.random.default_rng([seed, batch, 0xC4])

    def logu(lo, hi):
        return float(np.exp(r.uniform(np.log(lo), np.log(hi))))

    return [
        float(100000 - int(logu(1, 60000))),   # >($0, 100000): P(rank > k)
        float(1000 - int(logu(1, 30))),        # =($1, 1000):   P(rank = k)
        float(1000 - int(logu(2, 999))),       # <($2, 1000):   P(rank < k)
        float(int(r.integers(0, 1 << 30))),
        1000.0 - logu(1.005, 300.0),           # <($4, 1000.0)
        5000.0 - logu(1.5, 5000.0),            # >($5, 5000.0)
        100.0 - logu(1.005, 60.0),             # <($6, 100.0)
        float(r.uniform(-1e6, 1e6)),
    ]


def c4_batch_host(n: int, seed: int, batch: int) -> List[HostColumn]:
    """One C4 batch as numpy columns (seeded by (seed, batch))."""
    sh = c4_shifts(seed, batch)
    rng = np.random.default_rng([seed, batch, 1])
    cdf = _zipf_cdf()
    cols = []
    for j in range(8):
        rank = np.searchsorted(cdf, rng.random(n), side="right").astype(np.int64) + 1
        rank = np.minimum(rank, C4_ZIPF_MAX_RANK)
        if j < 4:
            cols.append(HostColumn(T.INT64, rank + np.int64(sh[j])))
        else:
            cols.append(HostColumn(T.FLOAT64, (rank.astype(np.float64) + rng.random(n)) + sh[j]))
    return cols


def c4_batch_device(n: int, seed: int, batch: int, device: str = "cuda"):
    """One C4 batch generated on the device (inverse-CDF Zipf sampling)."""
    import torch
    from .api import DeviceColumn
    sh = c4_shifts(seed, batch)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed) * 1_000_003 + int(batch))
    cdf = torch.from_numpy(_zipf_cdf()).to(device)
    cols = []
    for j in range(8):
        u = torch.rand(n, generator=gen, device=device, dtype=torch.float64)
        rank = torch.clamp(torch.searchsorted(cdf, u, right=True) + 1, max=C4_ZIPF_MAX_RANK)
        if j < 4:
            v = rank + int(sh[j])
        else:
            v = rank.to(torch.float64) + torch.rand(n, generator=gen, device=device, dtype=torch.float64) + sh[j]
        cols.append(DeviceColumn(T.INT64 if j < 4 else T.FLOAT64, v.contiguous().view(torch.uint8), None, 0, n))
    return cols


C2_LAST_DAY = 9861  # 1996-12-31 in days since 1970-01-01, the bound of C2_CONDITION


def c2_keep_mask(cols: Sequence[HostColumn]) -> np.ndarray:
    """Rows of a C2 table that pass C2_CONDITION ($2 valid, $4 valid and on or
    before 1996-12-31)."""
    return cols[2].valid() & cols[4].valid() & (cols[4].values() <= C2_LAST_DAY)


def c2_transcendental_rows(cols: Sequence[HostColumn]) -> np.ndarray:
    """For each output row of the C2 plan (the kept rows, in order): whether
    its first projection takes a CASE branch through LN ($5 NULL) or EXP
    ($5 = 0).  Only those rows' values come from CUDA's log / exp; every
    other row is exact binary64 arithmetic and must match bit for bit."""
    keep = c2_keep_mask(cols)
    v5, d5 = cols[5].valid()[keep], cols[5].values()[keep]
    return (~v5) | (d5 == 0)


def host_columns(name: str, n: int, seed: int = 1) -> List[HostColumn]:
    """Seeded numpy columns (CPU oracle, parity tests)."""
    return _np_columns(name, n, seed)


def _torch_mask(torch, gen, n: int, null_frac: float, device):
    """Bernoulli validity packed LSB-first into int32 words, padded to 64 B."""
    nwords = (n + 31) // 32
    padded = max(16, (nwords + 15) // 16 * 16)
    valid = torch.rand(padded * 32, generator=gen, device=device) >= null_frac
    valid[n:] = False
    bits = valid.view(padded, 32).to(torch.int64)
    weights = (torch.ones(32, dtype=torch.int64, device=device) << torch.arange(32, device=device))
    words = (bits * weights).sum(dim=1)
    words = torch.where(words >= (1 << 31), words - (1 << 32), words).to(torch.int32)
    return words.view(torch.uint8)


def device_columns(name: str, n: int, seed: int = 1, device: str = "cuda"):
    """Seeded columns generated on the device; returns a list of DeviceColumn."""
    import torch
    from .api import DeviceColumn
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)

    def u8(t):
        return t.contiguous().view(torch.uint8)

    cols = []
    if name == "c1":
        cols.append(DeviceColumn(T.INT64, u8(torch.randint(0, 1_000_000, (n,), generator=gen, device=device)), None, 0, n))
        cols.append(DeviceColumn(T.FLOAT64, u8(torch.randn(n, generator=gen, device=device, dtype=torch.float64)),
                                 None, 0, n))
        c2 = torch.randint(-1000, 1001, (n,), generator=gen, device=device, dtype=torch.int32)
        cols.append(DeviceColumn(T.INT32, u8(c2), _torch_mask(torch, gen, n, 0.10, device), 0, n))
        return cols
    if name == "c2":
        mk = lambda: _torch_mask(torch, gen, n, 0.05, device)  # noqa: E731
        cols.append(DeviceColumn(T.INT64, u8(torch.randint(0, 1 << 40, (n,), generator=gen, device=device)), mk(), 0, n))
        cols.append(DeviceColumn(T.INT64, u8(torch.randint(0, 1 << 40, (n,), generator=gen, device=device)), mk(), 0, n))
        cols.append(DeviceColumn(T.FLOAT64, u8(torch.randn(n, generator=gen, device=device, dtype=torch.float64) * 1e3),
                                 mk(), 0, n))
        cols.append(DeviceColumn(T.FLOAT64, u8(torch.randn(n, generator=gen, device=device, dtype=torch.float64) * 1e3),
                                 mk(), 0, n))
        d = torch.randint(DAY_1992_01_01, DAY_1992_01_01 + DAYS_7Y, (n,), generator=gen, device=device,
                          dtype=torch.int32)
        cols.append(DeviceColumn(T.TIMESTAMP_DAYS, u8(d), mk(), 0, n))
        cols.append(DeviceColumn(T.INT8, u8(torch.randint(0, 6, (n,), generator=gen, device=device, dtype=torch.int8)),
                                 mk(), 0, n))
        return cols
    if name == "c5":
        ri = lambda lo, hi, dt: torch.randint(lo, hi, (n,), generator=gen, device=device, dtype=dt)  # noqa: E731
        cols.append(DeviceColumn(T.INT32, u8(ri(1, 51, torch.int32)), None, 0, n))
        cols.append(DeviceColumn(T.INT64, u8(ri(90000, 10500001, torch.int64)), None, 0, n))
        cols.append(DeviceColumn(T.INT64, u8(ri(0, 11, torch.int64)), None, 0, n))
        cols.append(DeviceColumn(T.INT64, u8(ri(0, 9, torch.int64)), None, 0, n))
        cols.append(DeviceColumn(T.TIMESTAMP_DAYS, u8(ri(DAY_1992_01_01, DAY_1992_01_01 + DAYS_7Y, torch.int32)), None,
                                 0, n))
        cols.append(DeviceColumn(T.INT8, u8(ri(0, 3, torch.int8)), None, 0, n))
        cols.append(DeviceColumn(T.INT8, u8(ri(0, 2, torch.int8)), None, 0, n))
        return cols
    raise ValueError(name)


def device_to_host(cols) -> List[HostColumn]:
    """Copies DeviceColumns (or a row prefix of them) back to numpy HostColumns."""
    out = []
    for c in cols:
        dt = np_dtype(c.type_id)
        data = c.data.cpu().numpy().view(dt)[c.offset:c.offset + c.size].copy()
        mask = None if c.mask is None else c.mask.cpu().numpy().view(np.uint32).copy()
        out.append(HostColumn(c.type_id, data, mask, 0, c.size) if c.offset == 0 else
                   HostColumn(c.type_id, data, None, 0, c.size))
    return out
