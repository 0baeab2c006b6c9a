"""GPU parity at the full sizes of the hull and batched-world workloads.

* 20,000 convex hulls of 32 points (the hull stress workload): from the GPU's state after the
  drop has settled into a pile (300 steps), one open-loop pass of predict, aabbs, pairs and
  narrowphase (GJK, EPA, manifold refresh) on the GPU and on the oracle fed the same snapshot:
  pair sets and manifolds bit-identical.
* 4,096 batched worlds of 16..2,048 bodies (~1.7 M bodies): 16 sampled worlds, the largest
  among them, equal the same worlds stepped alone on the GPU and by the oracle (every world is
  one solver part, so the oracle's own colouring is the GPU's), bit for bit.
* The terrain workload (20,000 convex and 2,000 compound bodies on a 32,768-triangle mesh): from
  the GPU's state after 300 steps, one open-loop pass through the narrowphase (pairs with one key
  per compound child combination, the mesh pairs' triangle candidates) bit-identical to the
  oracle's, then one whole step in lockstep (the oracle fed the GPU's solver order)."""
import numpy as np
import pytest

from jbgpu import _abi, scenes, shard
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

pytestmark = pytest.mark.gpu


def test_hulls_20k_settled_pairs_and_narrowphase_open_loop(gpu_lib, oracle_lib):
    sc = scenes.hulls(20_000, seed=0)
    g = GpuWorld(sc)
    g.set_graph(True)
    for _ in range(300):
        g.step(sc.dt)
    c = g.counters()
    assert c["status_flags"] == 0
    assert c["contacts"] > 20_000 and c["epa_calls"] > 0, c      # a pile, not a free fall
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o)
    g.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    o.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    for st in (_abi.STAGE_PREDICT, _abi.STAGE_AABB, _abi.STAGE_PAIRS, _abi.STAGE_NARROWPHASE):
        g.stage(st, sc.dt)
        o.stage(st, sc.dt)
        if st == _abi.STAGE_AABB:
            assert not H.compare_state(o.get_state(), g.get_state(), fields=("aabb",))
        if st == _abi.STAGE_PAIRS:
            assert np.array_equal(o.get_pairs(), g.get_pairs())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    g.close()


def test_batched_4096_sampled_worlds_equal_solo_and_oracle(gpu_lib, oracle_lib):
    sc = scenes.batched_worlds(4096, seed=0)
    steps = 240
    rng = shard.world_body_ranges(sc)
    sizes = rng[:, 1] - rng[:, 0]
    pick = np.random.Generator(np.random.PCG64(1)).choice(len(sizes), 15, replace=False)
    sample = sorted(set(pick.tolist()) | {int(np.argmax(sizes))})
    big = GpuWorld(sc)
    big.set_graph(True)
    for _ in range(steps):
        big.step(sc.dt)
    assert big.counters()["status_flags"] == 0
    sb = big.get_state()
    big.close()
    for wi in sample:
        part = shard.subset_scene(sc, [wi])
        solo = GpuWorld(part)
        o = pyoracle.OracleWorld(part)
        for _ in range(steps):
            solo.step(sc.dt)
            o.step(sc.dt)
        ss, so = solo.get_state(), o.get_state()
        for k in ("transform", "linear_velocity", "angular_velocity", "activation_state"):
            assert np.array_equal(sb[k][rng[wi, 0]:rng[wi, 1]], ss[k]), (wi, k)
        assert not H.compare_state(so, ss), wi
        assert not H.compare_manifolds(o.get_manifolds(), solo.get_manifolds()), wi
        solo.close()


def test_terrain_20k_settled_narrowphase_and_step_lockstep(gpu_lib, oracle_lib):
    sc = scenes.SCENES["terrain_20k"]()
    g = GpuWorld(sc)
    for _ in range(300):
        g.step(sc.dt)
    c = g.counters()
    assert c["status_flags"] == 0
    assert c["contacts"] > 40_000 and c["gjk_calls"] > 100_000, c     # settled on the mesh
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o)
    g.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    o.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    for st in (_abi.STAGE_PREDICT, _abi.STAGE_AABB, _abi.STAGE_PAIRS, _abi.STAGE_NARROWPHASE):
        g.stage(st, sc.dt)
        o.stage(st, sc.dt)
        if st == _abi.STAGE_PAIRS:
            assert np.array_equal(o.get_pairs(), g.get_pairs())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    co, cg = o.counters(), g.counters()
    assert (co["gjk_calls"], co["epa_calls"]) == (cg["gjk_calls"], cg["epa_calls"])
    # one whole step more in lockstep: the GPU's solver order fed to the oracle
    H.copy_world(g, o)
    g.step(sc.dt)
    o.set_explicit_order(g.solver_order())
    o.step(sc.dt)
    assert o.counters()["status_flags"] == 0
    assert not H.compare_state(o.get_state(), g.get_state())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    g.close()
