"""Batched worlds split across GPUs, one process per GPU, with no collective on the data path.

Worlds of a batch are independent, so each rank steps only the worlds it owns.  These CPU
tests check the split (every world on exactly one rank, loads balanced by the greedy rule),
that per-world results of a world_size-2 gloo run of the oracle equal a single-rank run bit for
bit, and bench.py's host-side split and reductions under gloo.  The reference has no
counterpart (its dynamics world is single-threaded)."""
import multiprocessing as mp
import socket

import numpy as np
import pytest

import pyoracle
import shard_ranks
from jbgpu import scenes, shard


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _spawn(target, size, *args):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    ps = [ctx.Process(target=target, args=(r, size, port) + args + (q,)) for r in range(size)]
    for p in ps:
        p.start()
    try:
        res = q.get(timeout=240)
    finally:
        for p in ps:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in ps), [p.exitcode for p in ps]
    return res


@pytest.mark.parametrize("n_ranks", [2, 3, 4, 8])
def test_partition_covers_every_world_once_and_balances(n_ranks):
    counts = scenes.batched_world_counts(4096, seed=0)
    parts = shard.partition_worlds(counts, n_ranks)
    assert sorted(w for p in parts for w in p) == list(range(4096))
    for cost in ("square", "linear"):
        parts = shard.partition_worlds(counts, n_ranks, cost)
        loads = shard.rank_loads(counts, parts, cost)
        w = shard.world_costs(counts, cost)
        # list scheduling: the largest load is within (1 - 1/m) of one world's cost of the mean
        assert loads.max() <= loads.sum() / n_ranks + (1 - 1 / n_ranks) * w.max() + 1e-6
        assert loads.max() / loads.mean() < 1.01          # 4,096 worlds: near-perfect balance


def test_partition_small_cases():
    assert shard.partition_worlds([5, 1, 1, 1], 2, "linear") == [[0], [1, 2, 3]]
    assert shard.partition_worlds([3], 2) == [[0], []]
    with pytest.raises(ValueError):
        shard.partition_worlds([1, 2], 0)


def test_subset_scene_keeps_world_bodies_in_order():
    sc = scenes.batched_worlds(n_worlds=6, seed=4, nmin=16, nmax=40)
    rng = shard.world_body_ranges(sc)
    sub = shard.subset_scene(sc, [4, 1])
    assert sub.meta["worlds"] == [1, 4]
    want = np.concatenate([sc.bodies[rng[1, 0]:rng[1, 1]], sc.bodies[rng[4, 0]:rng[4, 1]]])
    assert np.array_equal(sub.bodies["transform"], want["transform"])
    assert list(np.unique(sub.bodies["world"])) == [0, 1]
    assert np.array_equal(sub.world_of_body, sub.bodies["world"])


def test_two_gloo_ranks_equal_one_rank_bit_for_bit(oracle_lib):
    kw = dict(n_worlds=7, seed=11, nmin=16, nmax=48)
    steps = 25
    parts, gathered = _spawn(shard_ranks.oracle_shard_rank, 2, kw, steps)
    assert sorted(w for p in parts for w in p) == list(range(7))
    merged = {}
    for per_world in gathered:
        assert not set(per_world) & set(merged)
        merged.update(per_world)
    sc = scenes.batched_worlds(**kw)
    o = pyoracle.OracleWorld(sc)
    for _ in range(steps):
        o.step(sc.dt)
    st = o.get_state()
    rng = shard.world_body_ranges(sc)
    for w in range(7):
        for k in shard_ranks.KEYS:
            assert np.array_equal(merged[w][k], st[k][rng[w, 0]:rng[w, 1]]), (w, k)


def test_bench_split_under_two_gloo_ranks():
    argv = ["--workload", "batched_4096", "--gpus", "2"]
    gathered, total, slowest = _spawn(shard_ranks.bench_split_rank, 2, argv)
    worlds = [g[0] for g in gathered]
    assert sorted(worlds[0] + worlds[1]) == list(range(4096)) and not set(worlds[0]) & set(worlds[1])
    sc = scenes.batched_worlds()
    assert total == sc.n_bodies
    assert slowest == 2.0
    assert all(g[2]["mode"] == "sharded by world" for g in gathered)
