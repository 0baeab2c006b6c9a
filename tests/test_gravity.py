"""DiscreteDynamicsWorld.setGravity and RigidBody.setGravity after bodies were added
(DiscreteDynamicsWorld.java:403-412, RigidBody.java:213-217): the library against the oracle,
closed loop, and through the mirror."""
import numpy as np
import pytest

from jbgpu import lib as jl, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

F = np.float32


@pytest.mark.gpu
def test_set_gravity_closed_loop_bit_exact(gpu_lib, oracle_lib):
    sc = scenes.small_mixed(60, seed=4)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    lifted = [5, 9]
    for s in range(sc.steps):
        for w in (o, g):
            if s == 40:
                w.set_gravity((2.0, -5.0, 0.5))
            if s == 90:
                w.set_body_gravity([3, 7, 11, 20], (0.0, 0.0, 0.0))
                w.set_body_gravity(lifted, [(0.0, 9.81, 0.0), (1.0, 4.0, -1.0)])
            if s == 150:
                w.set_gravity((0.0, -9.81, 0.0))
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
        if s == 149:
            up = g.get_state()["linear_velocity"][lifted, 1]
            assert np.all(up > 0.0), up        # the bodies given upward gravity rise
    with pytest.raises(jl.JbgpuError):
        g.set_body_gravity([len(sc.bodies)], (0.0, 0.0, 0.0))
    g.close()


@pytest.mark.gpu
def test_mirror_set_gravity_reads_like_the_reference(gpu_lib, oracle_lib):
    """World gravity changed after the first steps, one body's own gravity set after it was added
    (before and after the world's first step); the same calls on the oracle end bit-identical."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0))))
    shape = D.BoxShape((0.3, 0.3, 0.3))
    bodies = []
    for k in range(4):
        info = D.RigidBodyConstructionInfo(1.0, None, shape, shape.calculateLocalInertia(1.0))
        info.startWorldTransform = D.Transform(origin=(1.0 * k, 1.0, 0.0))
        b = D.RigidBody(info)
        b.setGravity((0.0, 50.0, 0.0))      # before addRigidBody: overridden by it
        world.addRigidBody(b)
        bodies.append(b)
    bodies[1].setGravity((0.0, -1.0, 0.0))  # after addRigidBody, before the first step: kept
    for _ in range(30):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    world.setGravity((0.0, -3.0, 1.0))
    bodies[2].setGravity((0.0, 2.0, 0.0))
    for _ in range(30):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    b = scenes._bodies(5)
    b["shape"] = [0, 1, 1, 1, 1]
    b["mass"] = [0.0, 1.0, 1.0, 1.0, 1.0]
    b["local_inertia"][1:] = shape.calculateLocalInertia(1.0)
    b["transform"][:, [0, 4, 8]] = 1.0
    b["transform"][1:, 9:] = np.array([[0, 1, 0], [1, 1, 0], [2, 1, 0], [3, 1, 0]], F)
    sc = scenes.Scene("mirror_gravity", 1.0 / 60.0, 60, {"gravity": (0.0, -9.81, 0.0)},
                      [D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0).desc(), shape.desc()], b)
    from jbgpu import _abi
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, -9.81, 0.0)))
    o.set_body_gravity([2], (0.0, -1.0, 0.0))
    for _ in range(30):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    o.set_gravity((0.0, -3.0, 1.0))
    o.set_body_gravity([3], (0.0, 2.0, 0.0))
    for _ in range(30):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    g = world._g
    assert not H.compare_state(o.get_state(), g.get_state())
    assert g.get_state()["linear_velocity"][3, 1] > F(0.0)   # the body given upward gravity rises
    world.close()
