"""GPU parity: the CUDA step against the oracle fed the same inputs and the same solver
order.  Open loop per stage from oracle snapshots (AABBs, pair set, narrowphase manifolds,
islands/sleeping, solver impulses and velocities, integration, activation), closed loop over
whole steps, and size-independent properties at the full 100k-body size.

Tolerances: the pair set, keys and manifold flags must be identical; floats are compared
bit for bit (the GPU kernels evaluate the reference's binary32 operations in the same order,
without contraction).  The looser bounds the reference parity contract allows (contacts
1e-5 relative, impulses/velocities 1e-4 relative) are asserted where a test says so."""
import numpy as np
import pytest

from jbgpu import _abi, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

pytestmark = pytest.mark.gpu

STAGES = [_abi.STAGE_PREDICT, _abi.STAGE_AABB, _abi.STAGE_PAIRS, _abi.STAGE_NARROWPHASE, _abi.STAGE_ISLANDS,
          _abi.STAGE_SOLVE, _abi.STAGE_INTEGRATE, _abi.STAGE_ACTIVATION]

SCENES = {
    "stack": lambda: scenes.box_stack(4),
    "mixed40": lambda: scenes.small_mixed(40, seed=1),
    "boxes300": lambda: scenes.boxes_on_plane(300, seed=2),
    "mixed120": lambda: scenes.small_mixed(120, seed=3),
    "hulls60": lambda: scenes.hulls(60, seed=4, box=8.0),
}


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("warm", [0, 45, 120])
def test_stage_by_stage_bit_exact(gpu_lib, oracle_lib, name, warm):
    sc = SCENES[name]()
    ref = pyoracle.OracleWorld(sc)
    for _ in range(warm):
        ref.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    H.copy_world(ref, o)
    H.copy_world(ref, g)
    o.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    g.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    for st in STAGES:
        H.copy_world(o, g)
        o.stage(st, sc.dt)
        g.stage(st, sc.dt)
        bs = H.compare_state(o.get_state(), g.get_state())
        bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
        assert not bs and not bm, (st, bs, bm)
        if st == _abi.STAGE_ISLANDS:
            a, b = o.get_state()["island_tag"], g.get_state()["island_tag"]
            assert same_partition(a, b)
        if st == _abi.STAGE_SOLVE:
            assert np.array_equal(o.solver_order(), g.solver_order())
    g.close()


def same_partition(a, b):
    """Island labels differ (the reference labels by union order), the grouping must not."""
    if not np.array_equal(a < 0, b < 0):
        return False
    m = a >= 0
    pairs = {}
    for x, y in zip(a[m], b[m]):
        if pairs.setdefault(x, y) != y:
            return False
    return len(set(pairs.values())) == len(pairs)


@pytest.mark.parametrize("name", list(SCENES))
def test_closed_loop_bit_exact(gpu_lib, oracle_lib, name):
    sc = SCENES[name]()
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    for s in range(150):
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    co, cg = o.counters(), g.counters()
    for k in ("pairs", "manifolds", "contacts", "solver_manifolds", "solver_rows", "colours", "gjk_calls", "epa_calls"):
        assert co[k] == cg[k], (k, co[k], cg[k])
    assert cg["status_flags"] == 0
    g.close()


@pytest.mark.parametrize("name", ["mixed120", "boxes300", "hulls60"])
@pytest.mark.parametrize("parts", [3, 16])
def test_range_parts_lockstep_bit_exact(gpu_lib, oracle_lib, name, parts):
    """Solver parts as ranges of the Morton leaf order, so that many manifolds are cut between
    parts and coloured grid-wide: each GPU step exports its solver order, the oracle steps in
    that order, and the two worlds stay bit-identical."""
    sc = SCENES[name]()
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc, config=_abi.default_config(**dict(sc.config, solver_parts=parts)))
    for s in range(120):
        g.step(sc.dt)
        order = g.solver_order()
        o.set_explicit_order(order)
        o.step(sc.dt)
        assert o.counters()["status_flags"] == 0, s   # the order covers exactly the oracle's manifolds
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    assert g.counters()["status_flags"] == 0
    g.close()


@pytest.mark.parametrize("name", ["stack", "mixed120", "boxes300"])
@pytest.mark.parametrize("parts", [0, 3])
@pytest.mark.parametrize("scope", [0, 1])
def test_residual_mode_bit_exact(gpu_lib, oracle_lib, name, parts, scope):
    """Residual-terminated PGS (tolerance 1e-4, at most 60 iterations): the GPU stops after the
    same iteration as the oracle fed its order, and state and manifolds stay bit-identical.
    parts 0: one solver part per world (block-local residual); 3: range parts, cut manifolds
    and a grid-wide residual.  scope 0: a residual per island; 1: one residual over the world's
    rows."""
    sc = SCENES[name]()
    cfg = dict(sc.config, solver_residual=1e-4, solver_max_iterations=60, solver_residual_scope=scope)
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(**cfg))
    g = GpuWorld(sc, config=_abi.default_config(**dict(cfg, solver_parts=parts)))
    iters = []
    for s in range(80):
        g.step(sc.dt)
        o.set_explicit_order(g.solver_order())
        o.step(sc.dt)
        co, cg = o.counters(), g.counters()
        assert co["status_flags"] == 0 and cg["status_flags"] == 0, s
        assert co["solver_iterations"] == cg["solver_iterations"], (s, co["solver_iterations"], cg["solver_iterations"])
        iters.append(cg["solver_iterations"])
        tr = g.residual_trace()
        assert len(tr) == cg["solver_iterations"], s
        if scope == 1 and len(tr) > 0:        # the trace holds the residual the stopping test saw
            n, tol = len(tr), np.float32(1e-4)
            r = tr[:, 0] / np.maximum(tr[:, 1], np.float32(1e-6))
            assert np.all(r[:n - 1] > tol), (s, r)
            if n < 60:                        # stopped by the test, not by the cap
                assert r[n - 1] <= tol, (s, r)
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    assert max(iters) > 10          # the tolerance, not the default 10 iterations, decided
    g.close()


def test_boxes_1k_300_steps_within_contract_tolerance(gpu_lib, oracle_lib):
    """The 1,000-box workload for its full 300 steps: per-step pair sets identical and
    body state within 1e-4 relative (the solver contract) of the oracle in colour order."""
    sc = scenes.boxes_on_plane(1000, seed=0)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    for s in range(sc.steps):
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 25 == 24:
            assert np.array_equal(o.get_pairs(), g.get_pairs()), s
            bs = H.compare_state(o.get_state(), g.get_state(), rtol=1e-4)
            assert not bs, (s, bs)
    g.close()


def test_step_simulation_accumulator(gpu_lib, oracle_lib):
    """stepSimulation(timeStep, maxSubSteps, fixedTimeStep): same substep counts and state."""
    sc = scenes.box_stack(3)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    for ts in [1 / 60, 1 / 45, 1 / 120, 1 / 30, 0.0, 1 / 60, 1 / 90] * 5:
        no = o.step_simulation(ts, 3, 1 / 60)
        ng = g.step_simulation(ts, 3, 1 / 60)
        assert no == ng
    assert not H.compare_state(o.get_state(), g.get_state())
    g.close()


def test_batched_worlds_equal_solo_runs(gpu_lib):
    """Bodies of different batch worlds never interact: stepping the batch equals stepping each
    world alone, bit for bit (every world has at most 2048 bodies, so each is one solver part
    and its manifolds are coloured the same way in the batch and alone)."""
    sc = scenes.batched_worlds(n_worlds=5, seed=3, nmin=16, nmax=120)
    big = GpuWorld(sc)
    counts = sc.meta["counts"]
    starts = np.concatenate([[0], np.cumsum(counts + 1)])
    solos = []
    for wi in range(5):
        part = scenes.Scene("w%d" % wi, sc.dt, sc.steps, sc.config, sc.shapes, sc.bodies[starts[wi]:starts[wi + 1]].copy())
        part.bodies["world"] = 0
        solos.append(GpuWorld(part))
    for _ in range(60):
        big.step(sc.dt)
        for s in solos:
            s.step(sc.dt)
    sb = big.get_state()
    for wi, s in enumerate(solos):
        ss = s.get_state()
        for k in ("transform", "linear_velocity", "angular_velocity", "activation_state"):
            assert np.array_equal(sb[k][starts[wi]:starts[wi + 1]], ss[k]), (wi, k)
        s.close()
    big.close()


@pytest.mark.parametrize("name", ["mixed120", "hulls60"])
def test_broadphase_refit_steps_keep_pairs_and_states(gpu_lib, oracle_lib, name):
    """Rebuilding the broadphase tree only every 5 steps (refitting it in between) finds the same
    pair sets as rebuilding it every step; with one solver part per world the states stay
    bit-identical too, and equal to the oracle's."""
    sc = SCENES[name]()
    a = GpuWorld(sc, config=_abi.default_config(**dict(sc.config, broadphase_rebuild_interval=1)))
    b = GpuWorld(sc, config=_abi.default_config(**dict(sc.config, broadphase_rebuild_interval=5)))
    o = pyoracle.OracleWorld(sc)
    for s in range(100):
        a.step(sc.dt)
        b.step(sc.dt)
        o.step(sc.dt)
        if s % 7 == 3:
            assert np.array_equal(a.get_pairs(), b.get_pairs()), s
            assert not H.compare_state(a.get_state(), b.get_state()), s
    assert not H.compare_state(o.get_state(), b.get_state())
    a.close()
    b.close()


@pytest.mark.parametrize("threads,smem", [(64, 512), (128, 64), (256, 0)])
def test_batched_worlds_independent_of_launch_shape(gpu_lib, threads, smem):
    """Threads per solver block and the shared-memory staging cap (the autotuner's knobs) change
    only scheduling: the batch steps to bit-identical states."""
    sc = scenes.batched_worlds(n_worlds=40, seed=5, nmin=16, nmax=600)
    ref = GpuWorld(sc)
    alt = GpuWorld(sc, config=_abi.default_config(**dict(sc.config, solver_threads=threads, solver_smem_bodies=smem)))
    for _ in range(40):
        ref.step(sc.dt)
        alt.step(sc.dt)
    assert not H.compare_state(ref.get_state(), alt.get_state())
    assert not H.compare_manifolds(ref.get_manifolds(), alt.get_manifolds())
    ref.close()
    alt.close()


def test_full_size_100k_solver_lockstep(gpu_lib, oracle_lib):
    """At the full 100k-body size (range solver parts, cut manifolds coloured grid-wide): from
    the GPU's settled state, three whole steps with the oracle fed the GPU's solver order stay
    bit-identical."""
    sc = scenes.mixed_100k(100_000, seed=0)
    g = GpuWorld(sc)
    for _ in range(400):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=True)
    for s in range(3):
        g.step(sc.dt)
        o.set_explicit_order(g.solver_order())
        o.step(sc.dt)
        assert o.counters()["status_flags"] == 0, s
        bs = H.compare_state(o.get_state(), g.get_state())
        bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
        assert not bs and not bm, (s, bs, bm)
    c = g.counters()
    assert c["status_flags"] == 0 and c["solver_manifolds"] > 20_000
    g.close()


def test_full_size_100k_pairs_and_properties(gpu_lib, oracle_lib):
    """At the full 100k-body size: the GPU pair set equals the oracle's (fed the GPU's body
    state), keys sorted and unique, manifolds hold 0..4 points within the breaking threshold,
    impulses non-negative and friction inside the cone, no non-finite state."""
    sc = scenes.mixed_100k(100_000, seed=0)
    g = GpuWorld(sc)
    for _ in range(120):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=True)
    o.stage(_abi.STAGE_PAIRS, sc.dt)
    g.stage(_abi.STAGE_PAIRS, sc.dt)
    kg, ko = g.get_pairs(), o.get_pairs()
    assert np.array_equal(kg, ko)
    assert np.all(np.diff(kg.astype(np.int64)) > 0)
    m = g.get_manifolds()
    assert m["num_points"].min() >= 0 and m["num_points"].max() <= 4
    mask = np.arange(4)[None, :] < m["num_points"][:, None]
    pts = m["points"][mask]
    assert np.all(pts[:, 15] <= 0.02 + 1e-7)                 # refreshContactPoints drops points beyond the threshold
    assert np.all(pts[:, 18] >= 0)                          # accumulated normal impulse clamp
    # friction inside the cone where the normal impulse is positive (the reference skips the
    # friction rows of a point whose normal impulse is zero, leaving its warm-started value)
    on = pts[:, 18] > 0
    fr = pts[on, 16] * pts[on, 18]
    assert np.all(np.abs(pts[on, 19]) <= fr * (1 + 1e-5) + 1e-6)
    st = g.get_state()
    for k in ("transform", "linear_velocity", "angular_velocity"):
        assert np.all(np.isfinite(st[k]))
    assert g.counters()["status_flags"] == 0
    g.close()


def test_full_size_100k_narrowphase_open_loop(gpu_lib, oracle_lib):
    """One narrowphase at full size from a shared snapshot: manifolds equal the oracle's."""
    sc = scenes.mixed_100k(100_000, seed=1)
    g = GpuWorld(sc)
    for _ in range(200):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o)
    g.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    o.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    for st in (_abi.STAGE_PREDICT, _abi.STAGE_AABB, _abi.STAGE_PAIRS, _abi.STAGE_NARROWPHASE):
        g.stage(st, sc.dt)
        o.stage(st, sc.dt)
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    g.close()
