"""Rank bodies for the world_size-2 gloo tests of tests/test_shard.py (spawned processes)."""
import os

import numpy as np

KEYS = ("transform", "linear_velocity", "angular_velocity", "activation_state")


def oracle_shard_rank(rank, size, port, scene_kwargs, steps, out_q):
    """One rank: its shard of a batched scene stepped by the oracle, per-world state gathered
    to rank 0 over gloo."""
    import torch.distributed as td
    import pyoracle
    from jbgpu import scenes, shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=size)
    try:
        sc = scenes.batched_worlds(**scene_kwargs)
        mine, parts = shard.shard_scene(sc, rank, size)
        o = pyoracle.OracleWorld(mine)
        for _ in range(steps):
            o.step(sc.dt)
        st = o.get_state()
        rng = shard.world_body_ranges(mine)
        per_world = {w: {k: st[k][rng[i, 0]:rng[i, 1]].copy() for k in KEYS} for i, w in enumerate(mine.meta["worlds"])}
        gathered = [None] * size
        td.all_gather_object(gathered, per_world)
        if rank == 0:
            out_q.put((parts, gathered))
    finally:
        td.destroy_process_group()


def bench_split_rank(rank, size, port, argv, out_q):
    """One rank of bench.py's host-side split: the scene each rank would step, and the rank-0
    reduction bench.py uses for the job's body count and its slowest rank's time."""
    import sys
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(size),
                      LOCAL_RANK=str(rank))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    sys.argv = ["bench.py"] + argv
    args = bench.parse()
    d = bench.Dist()
    try:
        sc, split = bench.rank_scene(args, d.rank, d.size)
        total = d.sum(sc.n_bodies)
        slowest = d.max(float(rank + 1))
        gathered = [None] * size
        d.td.all_gather_object(gathered, (sorted(sc.meta.get("worlds", [])), sc.n_bodies, split))
        if rank == 0:
            out_q.put((gathered, total, slowest))
    finally:
        d.close()
