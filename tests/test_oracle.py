"""CPU checks of the oracle (the CPU restatement of the reference's step).

The reference ships no tests, golden vectors or fixtures, and its Java code cannot run
here, so the oracle is pinned by internal consistency: the tree pair search equals the
SimpleBroadphase O(n^2) search (the reference's own simplest broadphase), GJK distances
equal analytic distances, runs are deterministic, and batched worlds equal solo worlds."""
import numpy as np
import pytest

from jbgpu import _abi, scenes

import pyoracle


@pytest.mark.parametrize("maker,steps", [(lambda: scenes.boxes_on_plane(400, seed=3), 40),
                                         (lambda: scenes.small_mixed(80, seed=5), 30)])
def test_tree_pairs_equal_all_pairs(oracle_lib, maker, steps):
    sc = maker()
    a = pyoracle.OracleWorld(sc)
    b = pyoracle.OracleWorld(sc)
    b.set_brute_force_pairs(True)
    for s in range(steps):
        a.step(sc.dt)
        b.step(sc.dt)
        pa, pb = a.get_pairs(), b.get_pairs()
        assert len(pa) == len(pb) and np.all(pa == pb), "step %d" % s
    assert len(pa) > sc.n_bodies - 1   # every body overlaps the plane


def _xf(pos, R=None):
    t = np.zeros(12, np.float32)
    t[:9] = (np.eye(3) if R is None else R).reshape(9)
    t[9:] = pos
    return t


SPHERE = lambda r: {"type": _abi.SHAPE_SPHERE, "params": (r, 0, 0, 0), "points": None}
BOX = lambda h: {"type": _abi.SHAPE_BOX, "params": (h, h, h, 0), "points": None}


@pytest.mark.parametrize("gap", [0.005, 0.01, 0.05])
def test_gjk_separated_spheres(oracle_lib, gap):
    # sphere-sphere through GJK (margins = radii): distance = |c0 - c1| - r0 - r1
    r0, r1 = 0.5, 0.3
    out = pyoracle.gjk(SPHERE(r0), _xf((0, 0, 0)), SPHERE(r1), _xf((r0 + r1 + gap, 0, 0)), 1.0)
    assert out[7] == 1
    assert abs(out[6] - gap) < 1e-5
    assert np.allclose(out[0:3], (-1, 0, 0), atol=1e-5)      # normal on B points from B to A


def test_gjk_box_box_face_contact(oracle_lib):
    # two unit boxes stacked along y, 0.01 apart: distance 0.01 along the y axis
    out = pyoracle.gjk(BOX(0.5), _xf((0, 1.01, 0)), BOX(0.5), _xf((0, 0, 0)), 1.0)
    assert out[7] == 1
    assert abs(out[6] - 0.01) < 1e-4
    assert np.allclose(out[0:3], (0, 1, 0), atol=1e-4)


def test_gjk_penetration_uses_epa(oracle_lib):
    # deep overlap of two boxes (cores intersect): EPA depth ~ 0.5 along an axis
    out = pyoracle.gjk(BOX(0.5), _xf((0, 0.5, 0)), BOX(0.5), _xf((0, 0, 0)), 1.0)
    assert out[7] == 1 and out[8] == 1
    assert abs(out[6] + 0.5) < 2e-3
    assert abs(abs(out[1]) - 1.0) < 1e-3


def test_integrate_transform_is_a_rotation(oracle_lib):
    rng = np.random.default_rng(0)
    R = scenes.random_rotations(rng, 1)[0]
    t = _xf((1, 2, 3), R)
    for ang in ([0, 0, 0], [1e-4, 0, 0], [0.3, -2.0, 1.5], [40.0, 0, 0]):
        out = pyoracle.integrate_transform(t, [1, 0, 0], ang, 1 / 60)
        B = out[:9].reshape(3, 3).astype(np.float64)
        assert np.allclose(B @ B.T, np.eye(3), atol=1e-5)
        assert abs(np.linalg.det(B) - 1) < 1e-5
        assert np.allclose(out[9:], [1 + 1 / 60, 2, 3], atol=1e-6)


def test_inertia_matches_generator(oracle_lib):
    shapes = [BOX(0.37), SPHERE(0.41), {"type": _abi.SHAPE_CAPSULE, "params": (0.25, 1.3, 0, 0), "points": None}]
    expect = [scenes.box_inertia(2.5, (0.37, 0.37, 0.37)), scenes.sphere_inertia(2.5, 0.41),
              scenes.capsule_inertia(2.5, 0.25, 1.3)]
    rng = np.random.default_rng(1)
    d = rng.standard_normal((32, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True)
    pts = (d * [0.3, 0.7, 0.5]).astype(np.float32)
    shapes.append({"type": _abi.SHAPE_CONVEX_HULL, "params": (0, 0, 0, 0), "points": pts})
    expect.append(scenes.hull_inertia(2.5, pts))
    for s, e in zip(shapes, expect):
        got = pyoracle.shape_local_inertia(s, 2.5)
        assert np.array_equal(got, np.asarray(e, np.float32)), (s["type"], got, e)


def test_deterministic(oracle_lib):
    sc = scenes.small_mixed(50, seed=11)
    a, b = pyoracle.OracleWorld(sc), pyoracle.OracleWorld(sc)
    for _ in range(40):
        a.step(sc.dt)
        b.step(sc.dt)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_boxes_come_to_rest_and_sleep(oracle_lib):
    sc = scenes.box_stack(3)
    w = pyoracle.OracleWorld(sc, order_mode=pyoracle.ORDER_REFERENCE)
    for _ in range(240):
        w.step(sc.dt)
    st = w.get_state()
    y = st["transform"][1:, 10]
    assert np.all(np.abs(y - np.round(y - 0.5) - 0.5) < 0.05)      # stacked at 0.5, 1.5, 2.5
    assert np.all(st["activation_state"][1:] == _abi.ISLAND_SLEEPING)   # 2 s below thresholds -> asleep


def test_reference_and_colour_orders_agree_statistically(oracle_lib):
    sc = scenes.boxes_on_plane(200, seed=4, steps=200)
    a = pyoracle.OracleWorld(sc, order_mode=pyoracle.ORDER_REFERENCE)
    b = pyoracle.OracleWorld(sc, order_mode=pyoracle.ORDER_COLOUR)
    for _ in range(200):
        a.step(sc.dt)
        b.step(sc.dt)
    ya, yb = a.get_state()["transform"][1:, 10], b.get_state()["transform"][1:, 10]
    assert abs(ya.mean() - yb.mean()) < 0.25
    assert ya.min() > 0.3 and yb.min() > 0.3                    # nothing sinks through the plane


def test_batched_worlds_equal_solo_worlds(oracle_lib):
    sc = scenes.batched_worlds(n_worlds=3, seed=2, nmin=16, nmax=40)
    big = pyoracle.OracleWorld(sc)
    counts = sc.meta["counts"]
    starts = np.concatenate([[0], np.cumsum(counts + 1)])
    solos = []
    for wi in range(3):
        part = scenes.Scene("w%d" % wi, sc.dt, sc.steps, sc.config, sc.shapes, sc.bodies[starts[wi]:starts[wi + 1]].copy())
        part.bodies["world"] = 0
        solos.append(pyoracle.OracleWorld(part))
    for _ in range(30):
        big.step(sc.dt)
        for s in solos:
            s.step(sc.dt)
    sb = big.get_state()
    for wi, s in enumerate(solos):
        ss = s.get_state()
        for k in ("transform", "linear_velocity", "angular_velocity"):
            assert np.array_equal(sb[k][starts[wi]:starts[wi + 1]], ss[k]), (wi, k)


def test_residual_mode_iterates_to_the_tolerance(oracle_lib):
    """Residual-terminated PGS: a loose tolerance stops after one iteration, tighter ones take
    more iterations (capped), and a fixed iteration count is unaffected by the cap."""
    sc = scenes.box_stack(4)
    warm = pyoracle.OracleWorld(sc)
    for _ in range(30):
        warm.step(sc.dt)
    its = {}
    for tol in (10.0, 1e-2, 1e-4, 1e-6):
        o = pyoracle.OracleWorld(sc, config=_abi.default_config(**dict(sc.config, solver_residual=tol,
                                                                          solver_max_iterations=150)))
        o.set_state(warm.get_state())
        o.set_manifolds(warm.get_manifolds())
        o.step(sc.dt)
        its[tol] = o.counters()["solver_iterations"]
    assert its[10.0] == 1
    assert its[10.0] <= its[1e-2] <= its[1e-4] <= its[1e-6] <= 150
    assert its[1e-4] > 10
    f = pyoracle.OracleWorld(sc)
    f.set_state(warm.get_state())
    f.set_manifolds(warm.get_manifolds())
    f.step(sc.dt)
    assert f.counters()["solver_iterations"] == sc.config["num_iterations"]
