"""The multi-GPU bench logic on CPU ranks (gloo, world size 2): programs are sharded over
the ranks by planned size with no exchange of data, every rank derives the same split on
its own, and a step's time is the slowest rank's.  (The NCCL launch of the same code is
not measured on this hardware: one GPU per machine here.)"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest


def test_shard_programs_balances_and_covers():
    from ptilopsis_gb300.batch import shard_programs
    rng = np.random.default_rng(7)
    sizes = np.clip(np.exp(np.log(22000) + 1.6 * rng.standard_normal(1000)), 1000, 500000).astype(int)
    for world in (1, 2, 3, 8):
        shards = shard_programs(sizes, world)
        flat = sorted(k for sh in shards for k in sh)
        assert flat == list(range(len(sizes)))
        loads = [int(sizes[sh].sum()) for sh in shards]
        # longest-first greedy: no shard exceeds the mean by more than the largest program
        assert max(loads) - sum(loads) / world <= sizes.max()
        assert all(sh == sorted(sh) for sh in shards)
    assert shard_programs([5, 5, 5, 5], 2) == [[0, 2], [1, 3]]
    assert shard_programs([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        shard_programs([1], 0)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, programs, out_dir):
    import json
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        mine = bench.rank_programs(programs, rank, world)
        everyone = [None] * world
        dist.all_gather_object(everyone, mine)
        # the slowest rank sets the step time
        slowest = bench.reduce_max(float(10 + rank), dist)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"mine": mine, "everyone": everyone, "slowest": slowest}, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_the_workload(tmp_path, built):
    import json
    import torch.multiprocessing as mp
    import bench
    programs, world = 48, 2
    mp.start_processes(_rank_main, args=(world, _free_port(), programs, str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    # every rank computed the same split, and its own share is its entry in it
    assert res[0]["everyone"] == res[1]["everyone"]
    for r in range(world):
        assert res[r]["mine"] == res[r]["everyone"][r]
        assert res[r]["slowest"] == 10.0 + world - 1
    a, b = (set(x) for x in res[0]["everyone"])
    assert not (a & b) and a | b == set(range(programs * world))
    # per-rank planned nodes within the largest program of each other (weak scaling)
    planned = [bench.planned_nodes(k) for k in range(programs * world)]
    loads = [sum(planned[k] for k in sh) for sh in res[0]["everyone"]]
    assert abs(loads[0] - loads[1]) <= max(planned)
    # one rank's share is what a one-rank run compiles of the same size class
    assert bench.rank_programs(programs, 0, 1) == list(range(programs))
