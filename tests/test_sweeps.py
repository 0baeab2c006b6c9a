"""Convex sweeps (CollisionWorld.convexSweepTest with a ClosestConvexResultCallback,
collision/dispatch/CollisionWorld.java:596-645, objectQuerySingle 391-490).

CPU: the oracle's restatement (GjkConvexCast conservative advancement) stops a falling sphere on a
box top and a box against a sphere where geometry says, within the cast's 0.001 distance
tolerance, takes the closest object, honours the filter, and marks sweeps that reach a static
plane (where the reference throws).  GPU: every field of every sweep's record is bit-identical to
the oracle's on the same bodies, for every convex cast shape, on mixed shapes after a simulated
drop, on batch worlds with per-sweep worlds and device buffers, and with plane sweeps marked."""
import numpy as np
import pytest

from jbgpu import _abi, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

F = np.float32


def _xf(rot, origin):
    t = np.zeros(12, F)
    t[:9] = np.asarray(rot, F).reshape(9)
    t[9:] = origin
    return t


def _quat_rows(q):
    x, y, z, w = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]], F)


def _sweeps(rng, n, lo, hi):
    """n (from, to) transform pairs: a third straight down from above, the rest between random
    points, each with its own start and end rotation."""
    a = rng.uniform(lo, hi, (n, 3)).astype(F)
    b = rng.uniform(lo, hi, (n, 3)).astype(F)
    a[: n // 3, 1] = hi[1] + 4.0
    b[: n // 3] = a[: n // 3]
    b[: n // 3, 1] = lo[1]
    fr = np.stack([_xf(_quat_rows(rng.normal(size=4)), a[i]) for i in range(n)])
    to = np.stack([_xf(_quat_rows(rng.normal(size=4)), b[i]) for i in range(n)])
    return fr, to


def _static_scene():
    shapes = [dict(scenes.PLANE),
              {"type": _abi.SHAPE_BOX, "params": (1.0, 1.0, 1.0, 0.0), "points": None},
              {"type": _abi.SHAPE_SPHERE, "params": (0.5, 0.0, 0.0, 0.0), "points": None}]
    b = np.concatenate([scenes._bodies(1) for _ in range(3)])
    b["shape"] = (0, 1, 2)
    b["transform"][0, 9:] = (0.0, -3.0, 0.0)
    b["transform"][1, 9:] = (0.0, 0.0, 0.0)
    b["transform"][2, 9:] = (5.0, 0.0, 0.0)
    b["collision_group"][1:] = 1           # static, but outside the static group the NO_PLANE mask drops
    return scenes.Scene("sweeps", 1.0 / 60.0, 1, {}, shapes, b)


NO_PLANE = ~2 & 0xFFFF      # a filter mask without the static group: the plane is never tested


def test_oracle_sweeps_stop_where_geometry_says(oracle_lib):
    o = pyoracle.OracleWorld(_static_scene())
    eye = np.eye(3, dtype=F)
    fr = np.stack([_xf(eye, (0, 10, 0)), _xf(eye, (5, 10, 0)), _xf(eye, (-10, 0.2, 0)), _xf(eye, (20, 10, 20))])
    to = np.stack([_xf(eye, (0, -1, 0)), _xf(eye, (5, -1, 0)), _xf(eye, (10, 0.2, 0)), _xf(eye, (20, 5, 20))])
    # a sphere of radius 0.5 (shape 2) onto the box top (y = 1) and onto the sphere (top y = 0.5)
    h, planes = o.convex_sweep(2, fr, to, mask=NO_PLANE)
    assert planes == 0 and list(h["body"]) == [1, 2, 1, -1]
    assert abs(h["fraction"][0] - 8.5 / 11.0) < 0.002 and np.allclose(h["normal"][0], (0, 1, 0), atol=1e-3)
    assert abs(h["fraction"][1] - 9.0 / 11.0) < 0.002 and np.allclose(h["normal"][1], (0, 1, 0), atol=1e-3)
    assert abs(h["fraction"][2] - 8.5 / 20.0) < 0.002 and np.allclose(h["normal"][2], (-1, 0, 0), atol=1e-3)
    assert abs(h["point"][0][1] - 1.0) < 0.01 and abs(h["point"][2][0] + 1.0) < 0.01
    assert h["fraction"][3] == 1.0 and np.all(h["normal"][3] == 0)
    # with the default filter the downward sweep past the box reaches the plane: marked -2
    h, planes = o.convex_sweep(2, fr, to)
    assert planes >= 2 and h["body"][0] == -2 and h["body"][1] == -2 and h["fraction"][0] == 1.0


def _same(a, b):
    return np.array_equal(a.view(np.uint8).reshape(len(a), -1), b.view(np.uint8).reshape(len(b), -1))


def _cast_shapes(sc):
    return [i for i, s in enumerate(sc.shapes) if s["type"] != _abi.SHAPE_STATIC_PLANE]


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [0, 60])
def test_gpu_sweeps_bit_exact_mixed(gpu_lib, oracle_lib, steps):
    sc = scenes.small_mixed(n=120, seed=13)
    g = GpuWorld(sc)
    for _ in range(steps):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=False)
    rng = np.random.Generator(np.random.PCG64(7))
    hits = 0
    for shape in _cast_shapes(sc):
        fr, to = _sweeps(rng, 256, np.array([-5, -1, -5], F), np.array([5, 9, 5], F))
        hg = g.convex_sweep_test(shape, fr, to, mask=NO_PLANE)
        ho, planes = o.convex_sweep(shape, fr, to, mask=NO_PLANE)
        assert planes == 0 and _same(ho, hg), (shape, np.nonzero(ho != hg)[0][:10])
        hits += (hg["body"] >= 0).sum()
        # the default filter: sweeps reaching the plane are marked on both sides
        hg = g.convex_sweep_test(shape, fr[:64], to[:64])
        ho, planes = o.convex_sweep(shape, fr[:64], to[:64])
        assert _same(ho, hg) and (hg["body"] == -2).sum() == planes > 0
    assert hits > 200
    g.close()


@pytest.mark.gpu
def test_gpu_sweeps_batched_worlds_and_device_buffers(gpu_lib, oracle_lib):
    torch = pytest.importorskip("torch")
    sc = scenes.hinged_chains(chains=3, links=4, loose=6, seed=8, worlds=4)
    g = GpuWorld(sc)
    for _ in range(30):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=False)
    rng = np.random.Generator(np.random.PCG64(10))
    fr, to = _sweeps(rng, 512, np.array([-4, 0, -4], F), np.array([4, 11, 4], F))
    world = rng.integers(0, 4, len(fr)).astype(np.int32)
    shape = _cast_shapes(sc)[0]
    hg = g.convex_sweep_test(shape, fr, to, world=world, mask=NO_PLANE)
    ho, _ = o.convex_sweep(shape, fr, to, world=world, mask=NO_PLANE)
    assert _same(ho, hg) and (hg["body"] >= 0).sum() > 20
    assert np.all(sc.bodies["world"][hg["body"][hg["body"] >= 0]] == world[hg["body"] >= 0])
    df = torch.from_numpy(fr).cuda()
    dt = torch.from_numpy(to).cuda()
    dw = torch.from_numpy(world).cuda()
    dh = torch.zeros(len(fr) * _abi.RAY_HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    g.convex_sweep_test_device(shape, df.data_ptr(), dt.data_ptr(), len(fr), dh.data_ptr(), world_ptr=dw.data_ptr(),
                               mask=NO_PLANE)
    g.synchronize()
    assert _same(hg, dh.cpu().numpy().view(_abi.RAY_HIT_DTYPE))
    g.close()


@pytest.mark.gpu
def test_gpu_sweep_api(gpu_lib):
    from jbgpu.lib import JbgpuError
    g = GpuWorld(_static_scene())
    assert len(g.convex_sweep_test(2, np.zeros((0, 12)), np.zeros((0, 12)))) == 0
    with pytest.raises(JbgpuError):
        g.convex_sweep_test(0, np.zeros((1, 12)), np.zeros((1, 12)))      # a plane is not a convex cast shape
    with pytest.raises(JbgpuError):
        g.convex_sweep_test(7, np.zeros((1, 12)), np.zeros((1, 12)))      # no such shape
    eye = np.eye(3, dtype=F)
    h = g.convex_sweep_test(2, [_xf(eye, (0, 10, 0))], [_xf(eye, (0, -1, 0))], mask=NO_PLANE)
    assert h["body"][0] == 1
    g.close()


@pytest.mark.gpu
def test_mirror_convex_sweep_test(gpu_lib):
    """convexSweepTest through the Python mirror, as the reference's callers write it."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    shape = D.BoxShape((0.5, 0.5, 0.5))
    info = D.RigidBodyConstructionInfo(0.0, None, shape)
    info.startWorldTransform = D.Transform(origin=(0.0, 0.0, 0.0))
    box = D.RigidBody(info)
    world.addRigidBody(box)
    world.stepSimulation(1.0 / 60.0)
    cast = D.SphereShape(0.25)
    cb = D.ClosestConvexResultCallback((0.0, 5.0, 0.0), (0.0, -5.0, 0.0))
    world.convexSweepTest(cast, D.Transform(origin=(0.0, 5.0, 0.0)), D.Transform(origin=(0.0, -5.0, 0.0)), cb)
    assert cb.hasHit() and cb.hitCollisionObject is box
    assert abs(cb.closestHitFraction - 4.25 / 10.0) < 0.002 and cb.hitNormalWorld[1] > 0.99
    miss = D.ClosestConvexResultCallback((3.0, 5.0, 0.0), (3.0, -5.0, 0.0))
    world.convexSweepTest(cast, D.Transform(origin=(3.0, 5.0, 0.0)), D.Transform(origin=(3.0, -5.0, 0.0)), miss)
    assert not miss.hasHit()
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), -3.0))))
    with pytest.raises(RuntimeError):
        world.convexSweepTest(cast, D.Transform(origin=(3.0, 5.0, 0.0)), D.Transform(origin=(3.0, -5.0, 0.0)), miss)
    world.close()


@pytest.mark.gpu
def test_gpu_sweeps_tree_walk_batch(gpu_lib, oracle_lib):
    """A batch large enough (at least 8 x SMs x 128 sweeps) to take the per-sweep tree walk instead
    of the (sweep, body) grid: the same records as the oracle."""
    sc = scenes.hinged_chains(chains=3, links=4, loose=6, seed=12, worlds=4)
    g = GpuWorld(sc)
    for _ in range(20):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=False)
    rng = np.random.Generator(np.random.PCG64(14))
    n = 200_000
    fr, to = _sweeps(rng, 2000, np.array([-4, 0, -4], F), np.array([4, 11, 4], F))
    fr, to = np.tile(fr, (n // 2000, 1)), np.tile(to, (n // 2000, 1))
    world = (np.arange(n) % 4).astype(np.int32)
    shape = _cast_shapes(sc)[-1]
    hg = g.convex_sweep_test(shape, fr, to, world=world, mask=NO_PLANE)
    ho, _ = o.convex_sweep(shape, fr, to, world=world, mask=NO_PLANE)
    assert _same(ho, hg) and (hg["body"] >= 0).sum() > 2000
    g.close()
