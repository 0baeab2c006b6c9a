"""CCD motion clamping in integrateTransforms (dynamics/DiscreteDynamicsWorld.java:679-739):
bodies whose predicted displacement exceeds their ccdMotionThreshold sweep a sphere of their
ccdSweptSphereRadius and stop at the first accepted time of impact.

CPU: the oracle's clamping stops the shots that tunnel through thin walls without it, and a
static plane on a sweep's path is flagged (the reference throws there).  GPU: the library's
clamping against the oracle, bit for bit - open loop from oracle snapshots, closed loop with and
without CUDA graphs - and the plane case reported as JBGPU_ERR_UNSUPPORTED."""
import numpy as np
import pytest

from jbgpu import _abi, scenes

import harness as H
import pyoracle

CCD_PLANE = 32   # status_flags bit: a CCD sweep reached a static plane


def _beyond(o, sc, x):
    first = sc.meta["ccd"]["bodies"][0]
    return int(np.sum(o.get_state()["transform"][first:, 9] > x))


def test_oracle_clamping_stops_tunnelling(oracle_lib):
    sc = scenes.ccd_shots(24, seed=1)
    bare = scenes.ccd_shots(24, seed=1)
    bare.meta["ccd"] = None
    o, b = pyoracle.OracleWorld(sc), pyoracle.OracleWorld(bare)
    swept = 0
    for _ in range(20):
        o.step(sc.dt)
        b.step(sc.dt)
        swept += o.counters()["ccd_clamped"]
        assert o.counters()["status_flags"] == 0
    wall = sc.meta["walls_x"][0] + 0.1
    assert _beyond(b, sc, wall) >= 15                 # without CCD most shots pass the first wall
    assert _beyond(o, sc, wall) <= _beyond(b, sc, wall) // 2
    assert swept > 100 and b.counters()["ccd_clamped"] == 0


def test_oracle_flags_a_sweep_that_reaches_a_static_plane(oracle_lib):
    sc = scenes.ccd_shots(8, seed=2, plane=True)
    o = pyoracle.OracleWorld(sc)
    o.step(sc.dt)
    assert o.counters()["status_flags"] & CCD_PLANE


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [0, 1])
def test_gpu_ccd_closed_loop_bit_exact(gpu_lib, oracle_lib, graph):
    from jbgpu.lib import GpuWorld
    sc = scenes.ccd_shots(24, seed=3)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    g.set_graph(bool(graph))
    for s in range(60):
        o.step(sc.dt)
        g.step(sc.dt)
        co, cg = o.counters(), g.counters()
        assert cg["status_flags"] == 0 and co["status_flags"] == 0, s
        assert co["ccd_clamped"] == cg["ccd_clamped"], (s, co["ccd_clamped"], cg["ccd_clamped"])
        if s % 6 == 5 or s < 4:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    assert _beyond(g, sc, sc.meta["walls_x"][0] + 0.1) <= 12
    if graph:
        held, err = g.graph_status()
        assert held > 0 and not err, err
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("warm", [0, 2, 3, 8, 25])
def test_gpu_ccd_integrate_stage_open_loop(gpu_lib, oracle_lib, warm):
    """The integrate stage alone from the oracle's state and manifolds after `warm` steps: the
    same clamped transforms (the touching-pair test reads those manifolds)."""
    from jbgpu.lib import GpuWorld
    sc = scenes.ccd_shots(24, seed=4)
    ref = pyoracle.OracleWorld(sc)
    for _ in range(warm):
        ref.step(sc.dt)
    o, g = pyoracle.OracleWorld(sc), GpuWorld(sc)
    H.copy_world(ref, o)
    H.copy_world(ref, g)
    for st in (_abi.STAGE_APPLY_GRAVITY, _abi.STAGE_PREDICT, _abi.STAGE_AABB, _abi.STAGE_PAIRS, _abi.STAGE_NARROWPHASE,
               _abi.STAGE_ISLANDS, _abi.STAGE_SOLVE):
        o.stage(st, sc.dt)
        g.stage(st, sc.dt)
    H.copy_world(o, g)
    o.stage(_abi.STAGE_INTEGRATE, sc.dt)
    g.stage(_abi.STAGE_INTEGRATE, sc.dt)
    assert o.counters()["ccd_clamped"] == g.counters()["ccd_clamped"] > 0
    assert not H.compare_state(o.get_state(), g.get_state())
    g.close()


@pytest.mark.gpu
def test_gpu_ccd_reports_a_static_plane_on_the_path(gpu_lib, oracle_lib):
    from jbgpu.lib import GpuWorld, JbgpuError
    sc = scenes.ccd_shots(8, seed=2, plane=True)
    g = GpuWorld(sc)
    with pytest.raises(JbgpuError) as e:
        g.step(sc.dt)
    assert e.value.code == _abi.ERR_UNSUPPORTED
    g.set_ccd(sc.meta["ccd"]["bodies"], 0.0, 0.0)     # CCD off: the same world steps again
    g.step(sc.dt)
    assert g.counters()["status_flags"] == 0
    with pytest.raises(JbgpuError):
        g.set_ccd([g.n_bodies], 1.0, 0.1)             # no such body
    g.close()


@pytest.mark.gpu
def test_mirror_bullet_stops_at_a_thin_wall(gpu_lib, oracle_lib):
    """The reference's usage through the Python mirror: a static thin box wall and a small sphere
    fired at 120 m/s (2 m per 1/60 s step, 20 times the wall's thickness) with
    setCcdMotionThreshold / setCcdSweptSphereRadius; a second sphere without CCD tunnels through.
    The oracle fed the same world agrees bit for bit."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, 0.0, 0.0))
    winfo = D.RigidBodyConstructionInfo(0.0, None, D.BoxShape((0.05, 2.0, 2.0)))
    winfo.startWorldTransform = D.Transform(origin=(5.0, 0.0, 0.0))
    world.addRigidBody(D.RigidBody(winfo))
    ball = D.SphereShape(0.1)
    shots = []
    for z, ccd in ((-1.0, True), (1.0, False)):
        info = D.RigidBodyConstructionInfo(0.1, None, ball, ball.calculateLocalInertia(0.1))
        info.startWorldTransform = D.Transform(origin=(0.0, 0.0, z))
        b = D.RigidBody(info)
        b.setLinearVelocity((120.0, 0.0, 0.0))
        if ccd:
            b.setCcdMotionThreshold(0.05)
            b.setCcdSweptSphereRadius(0.08)
        world.addRigidBody(b)
        shots.append(b)
    for _ in range(4):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    assert shots[0].getCenterOfMassTransform().origin[0] < 5.0     # stopped in front of the wall
    assert shots[1].getCenterOfMassTransform().origin[0] > 5.1     # tunnelled
    assert shots[0].getCcdSquareMotionThreshold() == np.float32(0.05) * np.float32(0.05)
    g = world._g
    sc = scenes.Scene("bullet", 1.0 / 60.0, 4, {"gravity": (0.0, 0.0, 0.0)},
                      [{"type": _abi.SHAPE_BOX, "params": (0.05, 2.0, 2.0, 0.0), "points": None},
                       {"type": _abi.SHAPE_SPHERE, "params": (0.1, 0.0, 0.0, 0.0), "points": None}],
                      np.concatenate([scenes._bodies(1), scenes._bodies(2)]))
    sc.bodies["shape"] = [0, 1, 1]
    sc.bodies["transform"][0, 9:] = (5.0, 0.0, 0.0)
    sc.bodies["transform"][1, 9:] = (0.0, 0.0, -1.0)
    sc.bodies["transform"][2, 9:] = (0.0, 0.0, 1.0)
    sc.bodies["mass"][1:] = 0.1
    sc.bodies["local_inertia"][1:] = ball.calculateLocalInertia(0.1)
    sc.bodies["linear_velocity"][1:] = (120.0, 0.0, 0.0)
    sc.meta["ccd"] = {"bodies": [1], "threshold": 0.05, "radius": 0.08}
    o = pyoracle.OracleWorld(sc)
    for _ in range(4):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    assert not H.compare_state(o.get_state(), g.get_state())
    world.close()
