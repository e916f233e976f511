"""Sharding by batch over ranks (world size 2, gloo on CPU).

Each rank evaluates its contiguous run of batches -- the oracle stands in for
the rank's GPU here -- the ranks exchange only their row counts, rank 0
collects the outputs, and their concatenation must equal the single-process
oracle result over the whole table (the filter is row-wise, so filtering the
batches one by one and concatenating is filtering the concatenation)."""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch.multiprocessing as mp

from blazingsql_gb300 import shard
from blazingsql_gb300 import workloads as W
from blazingsql_gb300.types import HostColumn, pack_validity


def test_shard_range_covers_every_batch_once():
    for nb in (0, 1, 5, 64, 513):
        for world in (1, 2, 3, 8):
            seen = [b for r in range(world) for b in shard.shard_range(nb, r, world)]
            assert seen == list(range(nb))
            sizes = [len(shard.shard_range(nb, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    assert shard.output_offsets([3, 0, 5, 2]) == [0, 3, 3, 8]


def _batches(sizes, seed=11):
    cols = W.host_columns("c2", sum(sizes), seed=seed)
    out, start = [], 0
    for n in sizes:
        part = []
        for c in cols:
            v = c.valid()[start:start + n]
            part.append(HostColumn(c.type_id, c.data[start:start + n].copy(), pack_validity(v)))
        out.append(part)
        start += n
    return cols, out


SIZES = [1, 31, 1000, 4097, 33, 0, 2500, 77]


def _rank_main(rank, world, port, result_path):
    import torch.distributed as dist
    from oracle import pyoracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _, batches = _batches(SIZES)

        def evaluate(batch):
            exp, rows = pyoracle.filter_project(batch, W.C2_CONDITION, W.C2_PROJECTIONS, 2, 0)
            return exp, rows

        local = shard.run_shard(batches, evaluate, rank, world)
        counts = shard.exchange_counts(local, len(batches))
        ordered = shard.collect(local, len(batches))
        if rank == 0:
            import pickle
            with open(result_path, "wb") as f:
                pickle.dump((counts, ordered), f)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_match_single_process_oracle():
    from oracle import pyoracle
    import pickle
    world = 2
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "r.pkl")
        mp.start_processes(_rank_main, args=(world, _free_port(), path), nprocs=world, join=True,
                           start_method="spawn")
        with open(path, "rb") as f:
            counts, ordered = pickle.load(f)
    full, batches = _batches(SIZES)
    exp, rows = pyoracle.filter_project(full, W.C2_CONDITION, W.C2_PROJECTIONS, 2, 0)
    assert sum(counts) == rows
    offsets = shard.output_offsets(counts)
    for j, e in enumerate(exp):
        vals = np.concatenate([o[j].values() for o in ordered])
        valid = np.concatenate([o[j].valid() for o in ordered])
        assert np.array_equal(valid, e.valid()), f"output {j}: validity"
        ev = e.values()
        assert np.array_equal(vals[valid].view(np.uint8), ev[e.valid()].view(np.uint8)), f"output {j}: values"
        for b, off in enumerate(offsets):  # each batch's rows start at its offset
            n = counts[b]
            assert np.array_equal(ordered[b][j].valid(), e.valid()[off:off + n])
