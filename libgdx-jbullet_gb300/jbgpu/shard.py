"""Splitting a batch of independent worlds across GPUs (one process per GPU).

Worlds of a batch never interact, so a batch shards by world with no collective on the data
path: each rank builds its own jbgpu_world from the worlds it owns and steps it alone; only
counters and timings meet on the host.  The reference has no counterpart (its
DiscreteDynamicsWorld is single-threaded and `setNumTasks` is a no-op,
dynamics/DiscreteDynamicsWorld.java:1084-1085).

The split is a greedy longest-processing-time assignment: worlds in decreasing cost order,
each to the rank with the least cost so far (ties to the lower rank).  The default cost of a
world of N bodies is N^2, a bound on its pair and colouring work in a pile; `cost="linear"`
balances body counts instead.  Greedy LPT ends within 4/3 of the best possible maximum load and
within one world's cost of the mean load.
"""
import numpy as np

from .scenes import Scene


def world_costs(counts, cost="square"):
    c = np.asarray(counts, np.float64)
    if cost == "square":
        return c * c
    if cost == "linear":
        return c
    raise ValueError("cost must be 'square' or 'linear'")


def partition_worlds(counts, n_ranks, cost="square"):
    """World indices per rank (each list ascending); every world goes to exactly one rank."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be at least 1")
    w = world_costs(counts, cost)
    order = sorted(range(len(w)), key=lambda i: (-w[i], i))
    load = np.zeros(n_ranks)
    owned = [[] for _ in range(n_ranks)]
    for i in order:
        r = int(np.argmin(load))          # first minimum: ties go to the lower rank
        owned[r].append(i)
        load[r] += w[i]
    return [sorted(o) for o in owned]


def rank_loads(counts, parts, cost="square"):
    w = world_costs(counts, cost)
    return np.array([w[p].sum() if len(p) else 0.0 for p in parts])


def world_body_ranges(scene):
    """(start, end) body index of every world of a batched scene (bodies are stored world after
    world, each world's plane first)."""
    wob = scene.world_of_body
    if wob is None:
        return np.array([[0, scene.n_bodies]])
    nw = int(wob.max()) + 1
    starts = np.searchsorted(wob, np.arange(nw), side="left")
    ends = np.searchsorted(wob, np.arange(nw), side="right")
    if not np.all(np.diff(wob) >= 0):
        raise ValueError("bodies of a batched scene must be stored world after world")
    return np.stack([starts, ends], 1)


def subset_scene(scene, worlds):
    """The batch of the given worlds only (in ascending world order), renumbered 0..k-1; shapes
    are shared, joints are not supported (batched scenes here carry none)."""
    if scene.meta.get("joints"):
        raise ValueError("sharding a batch with joints is not supported")
    worlds = sorted(int(x) for x in worlds)
    rng = world_body_ranges(scene)
    idx = np.concatenate([np.arange(rng[w, 0], rng[w, 1]) for w in worlds]) if worlds else np.zeros(0, int)
    b = scene.bodies[idx].copy()
    wob = np.concatenate([np.full(rng[w, 1] - rng[w, 0], k, np.int32) for k, w in enumerate(worlds)]) \
        if worlds else np.zeros(0, np.int32)
    b["world"] = wob
    meta = dict(scene.meta)
    meta["worlds"] = worlds
    if "counts" in meta:
        meta["counts"] = np.asarray(scene.meta["counts"])[worlds]
    return Scene("%s_shard%d" % (scene.name, len(worlds)), scene.dt, scene.steps, scene.config, scene.shapes, b,
                 world_of_body=wob, meta=meta)


def shard_scene(scene, rank, n_ranks, cost="square"):
    """This rank's share of a batched scene."""
    rng = world_body_ranges(scene)
    counts = rng[:, 1] - rng[:, 0]
    parts = partition_worlds(counts, n_ranks, cost)
    return subset_scene(scene, parts[rank]), parts
