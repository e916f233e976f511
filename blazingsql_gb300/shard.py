"""Batches of one plan spread over ranks (one process per GPU).

Rows are independent, so the evaluator shards by batch with no exchange of
data between ranks: each rank takes a contiguous run of the execution graph's
batches (as the reference runs many batches at once on its executor threads,
engine/src/execution_graph/executor.cpp:217-255), evaluates them on its own
GPU, and the only thing the ranks share is host-side bookkeeping: each batch's
output row count, from which every batch's offset in the concatenated result
follows.  ``torch.distributed`` (any backend; gloo on the host) carries the
counts, and optionally the outputs themselves when rank 0 collects them.
"""
from __future__ import annotations

from typing import Callable, List, Optional, Sequence, Tuple


def shard_range(num_batches: int, rank: int, world: int) -> range:
    """The contiguous run of batch indices rank ``rank`` of ``world`` takes:
    batch counts differ by at most one between ranks, lower ranks first."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(num_batches, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def output_offsets(row_counts: Sequence[int]) -> List[int]:
    """Exclusive prefix sums: where each batch's rows start in the
    concatenation of all batches' outputs (in batch order)."""
    out, acc = [], 0
    for r in row_counts:
        out.append(acc)
        acc += int(r)
    return out


def run_shard(batches: Sequence, evaluate: Callable, rank: int, world: int) -> List[Tuple[int, object, int]]:
    """Evaluates this rank's batches in order: [(batch index, result, rows)],
    ``evaluate(batch) -> (result, rows)`` (for the GPU path: a compiled plan's
    execute, or a batch runner over the shard's batches)."""
    out = []
    for b in shard_range(len(batches), rank, world):
        res, rows = evaluate(batches[b])
        out.append((b, res, int(rows)))
    return out


def exchange_counts(local: Sequence[Tuple[int, object, int]], num_batches: int, group=None) -> List[int]:
    """Every batch's output row count on every rank (an all-gather of the
    local counts over torch.distributed)."""
    import torch.distributed as dist
    mine = [(b, rows) for b, _, rows in local]
    parts: List[Optional[list]] = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, mine, group=group)
    counts = [-1] * num_batches
    for part in parts:
        for b, rows in part:
            counts[b] = rows
    if any(c < 0 for c in counts):
        raise RuntimeError("a batch was evaluated by no rank")
    return counts


def collect(local: Sequence[Tuple[int, object, int]], num_batches: int, dst: int = 0, group=None):
    """Rank ``dst`` receives every batch's result in batch order (host
    objects, e.g. HostColumn lists); other ranks receive None."""
    import torch.distributed as dist
    parts: Optional[List[Optional[list]]] = [None] * dist.get_world_size(group) if dist.get_rank(group) == dst else None
    dist.gather_object([(b, res) for b, res, _ in local], parts, dst=dst, group=group)
    if parts is None:
        return None
    ordered: List[object] = [None] * num_batches
    for part in parts:
        for b, res in part:
            ordered[b] = res
    return ordered
