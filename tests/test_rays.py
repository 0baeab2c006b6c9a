"""Ray queries (CollisionWorld.rayTest with a ClosestRayResultCallback,
collision/dispatch/CollisionWorld.java:553-591, rayTestSingle 260-331).

CPU: the oracle's restatement hits boxes, spheres and the plane where geometry says (within the
conservative-advancement tolerance of SubsimplexConvexCast: the cast stops within 0.01 of the
surface), takes the closest object, honours the callback's filter and reports misses as the
reference's callback leaves them.  GPU: every field of every ray's hit record is bit-identical to
the oracle's on the same bodies (the GPU's transforms copied into the oracle): mixed shapes after
a simulated drop, batch worlds with per-ray worlds, device buffers, and overlapping objects that
send rays through the in-order replay."""
import numpy as np
import pytest

from jbgpu import _abi, scenes
from jbgpu.lib import GpuWorld, JbgpuError

import harness as H
import pyoracle

F = np.float32


def _scene_for_rays():
    shapes = [dict(scenes.PLANE),
              {"type": _abi.SHAPE_BOX, "params": (1.0, 1.0, 1.0, 0.0), "points": None},
              {"type": _abi.SHAPE_SPHERE, "params": (1.0, 0.0, 0.0, 0.0), "points": None}]
    b = np.concatenate([scenes._bodies(1) for _ in range(4)])
    b["shape"] = (0, 1, 2, 1)
    b["transform"][0, 9:] = (0.0, -3.0, 0.0)
    b["transform"][1, 9:] = (0.0, 0.0, 0.0)
    b["transform"][2, 9:] = (5.0, 0.0, 0.0)
    b["transform"][3, 9:] = (0.0, 0.0, 6.0)
    b["collision_group"][3] = 4            # only rays whose mask includes 4 see body 3
    return scenes.Scene("rays", 1.0 / 60.0, 1, {}, shapes, b)


def test_oracle_rays_hit_where_geometry_says(oracle_lib):
    o = pyoracle.OracleWorld(_scene_for_rays())
    frm = np.array([[0, 10, 0], [5, 10, 0], [20, 10, 0], [30, 10, 30], [0, 10, 6], [-10, 0.5, 0]], F)
    to = np.array([[0, -10, 0], [5, -10, 0], [20, -10, 0], [30, 5, 30], [0, -10, 6], [10, 0.5, 0]], F)
    h = o.ray_test(frm, to)
    assert list(h["body"]) == [1, 2, 0, -1, 3, 1]
    # box top at y = 1, sphere top at y = 1: entry 9/20, the cast stopping up to 0.01 before it
    for k in (0, 1):
        assert 0.45 - 0.01 / 20 - 1e-6 <= h["fraction"][k] <= 0.45 + 1e-6
        assert np.allclose(h["normal"][k], (0, 1, 0), atol=1e-3)
        assert np.allclose(h["point"][k], frm[k] + h["fraction"][k] * (to[k] - frm[k]), atol=1e-5)
    assert abs(h["fraction"][2] - 13.0 / 20.0) < 1e-6            # the plane y = -3, exactly by triangle
    assert h["normal"][2][1] > 0 and abs(h["normal"][2][0]) < 1e-6 * abs(h["normal"][2][1])
    assert h["fraction"][3] == 1.0 and np.all(h["point"][3] == 0) and np.all(h["normal"][3] == 0)
    # body 3 is group 4: the default mask (-1) sees it, a mask without 4 does not
    assert o.ray_test(frm[4:5], to[4:5])["body"][0] == 3
    assert o.ray_test(frm[4:5], to[4:5], mask=~4)["body"][0] == 0
    # every body here is static, and a static body's default mask leaves out the static group
    assert o.ray_test(frm[4:5], to[4:5], group=2)["body"][0] == -1
    # a ray crossing the box sideways at y = 0.5 enters at x = -1
    assert abs(h["fraction"][5] - 9.0 / 20.0) <= 0.01 / 20 + 1e-6
    assert np.allclose(h["normal"][5], (-1, 0, 0), atol=1e-3)


def _rays(rng, n, lo, hi):
    a = rng.uniform(lo, hi, (n, 3)).astype(F)
    b = rng.uniform(lo, hi, (n, 3)).astype(F)
    a[: n // 4, 1] = hi[1] + 5.0                         # a quarter straight down from above
    b[: n // 4] = a[: n // 4]
    b[: n // 4, 1] = -2.0
    return a, b


def _same(o_hits, g_hits):
    return np.array_equal(o_hits.view(np.uint8).reshape(len(o_hits), -1), g_hits.view(np.uint8).reshape(len(g_hits), -1))


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [0, 90])
def test_gpu_rays_bit_exact_mixed(gpu_lib, oracle_lib, steps):
    sc = scenes.small_mixed(n=120, seed=11)
    g = GpuWorld(sc)
    for _ in range(steps):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=False)
    rng = np.random.Generator(np.random.PCG64(5))
    frm, to = _rays(rng, 4096, np.array([-5, -1, -5], F), np.array([5, 10, 5], F))
    hg = g.ray_test(frm, to)
    ho = o.ray_test(frm, to)
    assert _same(ho, hg), np.nonzero(ho != hg)[0][:10]
    assert (hg["body"] >= 0).sum() > 1000 and (hg["body"] == 0).sum() > 10
    # the filter: static bodies only (the plane)
    hs = g.ray_test(frm[:512], to[:512], group=1, mask=2)
    assert _same(o.ray_test(frm[:512], to[:512], group=1, mask=2), hs)
    assert set(np.unique(hs["body"])) <= {-1, 0}
    g.close()


@pytest.mark.gpu
def test_gpu_rays_batched_worlds_and_device_buffers(gpu_lib, oracle_lib):
    torch = pytest.importorskip("torch")
    sc = scenes.hinged_chains(chains=3, links=4, loose=6, seed=6, worlds=4)
    g = GpuWorld(sc)
    for _ in range(30):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=False)
    rng = np.random.Generator(np.random.PCG64(9))
    frm, to = _rays(rng, 2048, np.array([-4, 0, -4], F), np.array([4, 12, 4], F))
    world = rng.integers(0, 4, len(frm)).astype(np.int32)
    hg = g.ray_test(frm, to, world=world)
    assert _same(o.ray_test(frm, to, world=world), hg)
    assert np.all(sc.bodies["world"][hg["body"][hg["body"] >= 0]] == world[hg["body"] >= 0])
    # the same rays from device buffers
    df = torch.from_numpy(frm).cuda()
    dt = torch.from_numpy(to).cuda()
    dw = torch.from_numpy(world).cuda()
    dh = torch.zeros(len(frm) * _abi.RAY_HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    g.ray_test_device(df.data_ptr(), dt.data_ptr(), len(frm), dh.data_ptr(), world_ptr=dw.data_ptr())
    g.synchronize()
    hd = dh.cpu().numpy().view(_abi.RAY_HIT_DTYPE)
    assert _same(hg, hd)
    # a world id outside the batch: rejected before any work from host buffers; from device
    # buffers the ray finds nothing and the call reports the bad id
    bad = world.copy()
    bad[7] = 4
    with pytest.raises(JbgpuError) as e:
        g.ray_test(frm, to, world=bad)
    assert e.value.code == _abi.ERR_INVALID_ARGUMENT
    dw.copy_(torch.from_numpy(bad))
    with pytest.raises(JbgpuError) as e:
        g.ray_test_device(df.data_ptr(), dt.data_ptr(), len(frm), dh.data_ptr(), world_ptr=dw.data_ptr())
    assert e.value.code == _abi.ERR_INVALID_ARGUMENT
    g.synchronize()
    hb = dh.cpu().numpy().view(_abi.RAY_HIT_DTYPE)
    assert hb["body"][7] == -1
    keep = np.arange(len(frm)) != 7
    assert _same(hg[keep], hb[keep])
    # and the next call with good ids succeeds again (the flag belongs to one call)
    dw.copy_(torch.from_numpy(world))
    g.ray_test_device(df.data_ptr(), dt.data_ptr(), len(frm), dh.data_ptr(), world_ptr=dw.data_ptr())
    g.synchronize()
    assert _same(hg, dh.cpu().numpy().view(_abi.RAY_HIT_DTYPE))
    g.close()


@pytest.mark.gpu
def test_gpu_rays_replayed_in_body_order(gpu_lib, oracle_lib):
    """The in-order replay (the reference's object loop, a block per ray) that takes the rays the
    tree walk cannot decide, forced for every ray: the same records as the tree walk and the
    oracle, on overlapping static spheres a few micrometres apart and on the mixed scene."""
    shapes = [{"type": _abi.SHAPE_SPHERE, "params": (1.0, 0.0, 0.0, 0.0), "points": None}]
    k = 64
    b = np.concatenate([scenes._bodies(1) for _ in range(2 * k)])
    b["shape"] = 0
    for i in range(k):
        b["transform"][2 * i, 9:] = (3.0 * i, 0.0, 0.0)
        b["transform"][2 * i + 1, 9:] = (3.0 * i, 2e-6 * (i % 5), 0.0)
    rng = np.random.Generator(np.random.PCG64(3))
    xs = np.repeat(3.0 * np.arange(k), 16) + rng.uniform(-0.05, 0.05, 16 * k)
    frm = np.stack([xs, np.full_like(xs, 10.0), rng.uniform(-0.05, 0.05, 16 * k)], 1).astype(F)
    to = frm.copy()
    to[:, 1] = -10.0
    mixed = scenes.small_mixed(n=120, seed=12)
    mf, mt = _rays(rng, 2048, np.array([-5, -1, -5], F), np.array([5, 10, 5], F))
    for sc, fr_, to_ in ((scenes.Scene("spheres", 1.0 / 60.0, 1, {}, shapes, b), frm, to), (mixed, mf, mt)):
        g = GpuWorld(sc)
        o = pyoracle.OracleWorld(sc)
        fast = g.ray_test(fr_, to_)
        g.set_ray_replay(True)
        slow = g.ray_test(fr_, to_)
        assert g.counters()["ray_replays"] == len(fr_)
        assert _same(fast, slow) and _same(o.ray_test(fr_, to_), slow)
        g.close()


@pytest.mark.gpu
def test_gpu_ray_api(gpu_lib):
    from jbgpu.lib import JbgpuError
    sc = _scene_for_rays()
    g = GpuWorld(sc)
    assert len(g.ray_test(np.zeros((0, 3)), np.zeros((0, 3)))) == 0
    with pytest.raises(JbgpuError):
        g.ray_test(np.zeros((2, 3)), np.ones((2, 3)), world=[0, 3])     # no such batch world
    h = g.ray_test([[0, 10, 0]], [[0, -10, 0]])
    assert h["body"][0] == 1
    g.close()


@pytest.mark.gpu
def test_mirror_ray_test(gpu_lib):
    """rayTest through the Python mirror, as the reference's callers write it."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0))))
    shape = D.BoxShape((0.5, 0.5, 0.5))
    info = D.RigidBodyConstructionInfo(1.0, None, shape, shape.calculateLocalInertia(1.0))
    info.startWorldTransform = D.Transform(origin=(0.0, 3.0, 0.0))
    box = D.RigidBody(info)
    world.addRigidBody(box)
    for _ in range(5):
        world.stepSimulation(1.0 / 60.0)
    cb = D.ClosestRayResultCallback((0.0, 10.0, 0.0), (0.0, -10.0, 0.0))
    world.rayTest(cb.rayFromWorld, cb.rayToWorld, cb)
    assert cb.hasHit() and cb.collisionObject is box
    top = box.getCenterOfMassTransform().origin[1] + 0.5
    assert abs(cb.hitPointWorld[1] - top) < 0.02 and cb.hitNormalWorld[1] > 0.99
    miss = D.ClosestRayResultCallback((5.0, 10.0, 0.0), (5.0, 1.0, 0.0))
    world.rayTest(miss.rayFromWorld, miss.rayToWorld, miss)
    assert not miss.hasHit() and miss.closestHitFraction == 1.0
    world.close()
