"""DiscreteDynamicsWorld.removeRigidBody (CollisionWorld.removeCollisionObject,
collision/dispatch/CollisionWorld.java:157-176): the library against the oracle after bodies
(a static plane among them) leave a settling world and new ones join it, closed loop; refusal of
a body a joint uses; the mirror's removeRigidBody."""
import numpy as np
import pytest

from jbgpu import _abi, lib as jl, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

F = np.float32


def _newcomers(sc, k, seed):
    """k copies of the scene's dynamic bodies (same shapes, masses, inertias) dropped over its
    middle at rest."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dyn = np.nonzero(sc.bodies["mass"] > 0)[0]
    b = sc.bodies[rng.choice(dyn, k, replace=False)].copy()
    b["transform"][:, 9:] = np.stack([rng.uniform(-2, 2, k), rng.uniform(4, 7, k), rng.uniform(-2, 2, k)], 1).astype(F)
    b["linear_velocity"] = 0.0
    b["angular_velocity"] = 0.0
    return scenes.Scene("newcomers", sc.dt, 0, {}, [], b)


def _compare(o, g, tag):
    bs = H.compare_state(o.get_state(), g.get_state())
    bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    assert not bs and not bm, (tag, bs, bm)
    assert np.array_equal(o.get_pairs(), g.get_pairs()), tag


@pytest.mark.gpu
def test_remove_and_add_bodies_closed_loop_bit_exact(gpu_lib, oracle_lib):
    sc = scenes.small_mixed(90, seed=6)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    for s in range(60):
        o.step(sc.dt)
        g.step(sc.dt)
    _compare(o, g, "before")
    gone = [3, 10, 11, 40, 89]          # bodies in the pile, the last one added
    for w in (o, g):
        w.remove_bodies(gone)
    assert g.n_bodies == o.n_bodies == len(sc.bodies) - len(gone)
    _compare(o, g, "removed")
    for s in range(60):
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9:
            _compare(o, g, s)
    new = _newcomers(sc, 6, 2)
    o.add_scene(new)
    g.add_scene(new)
    for w in (o, g):
        w.remove_bodies([0])            # the static plane: every pair with it goes
    for s in range(90):
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9:
            _compare(o, g, 100 + s)
    assert g.counters()["status_flags"] == 0
    with pytest.raises(jl.JbgpuError):
        g.remove_bodies([1, 1])
    with pytest.raises(jl.JbgpuError):
        g.remove_bodies([g.n_bodies])
    g.close()


@pytest.mark.gpu
def test_remove_refuses_a_jointed_body(gpu_lib, oracle_lib):
    sc = scenes.jointed_chains(seed=1)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    a = int(sc.meta["joints"][0]["a"])
    with pytest.raises(jl.JbgpuError):
        g.remove_bodies([a])
    with pytest.raises(ValueError):
        o.remove_bodies([a])
    g.close()


@pytest.mark.gpu
def test_mirror_remove_rigid_body_reads_like_the_reference(gpu_lib, oracle_lib):
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0))))
    shape = D.BoxShape((0.3, 0.3, 0.3))
    bodies = []
    for k in range(6):
        info = D.RigidBodyConstructionInfo(1.0, None, shape, shape.calculateLocalInertia(1.0))
        info.startWorldTransform = D.Transform(origin=(0.1 * k, 0.4 + 0.65 * k, 0.0))
        b = D.RigidBody(info)
        world.addRigidBody(b)
        bodies.append(b)
    for _ in range(40):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    world.removeRigidBody(bodies[2])     # the stack above it falls
    assert bodies[3]._index == 3 and world.getNumCollisionObjects() == 6
    for _ in range(40):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    b = scenes._bodies(7)
    b["shape"] = [0] + [1] * 6
    b["mass"] = [0.0] + [1.0] * 6
    b["local_inertia"][1:] = shape.calculateLocalInertia(1.0)
    b["transform"][:, [0, 4, 8]] = 1.0
    b["transform"][1:, 9:] = np.array([[0.1 * k, 0.4 + 0.65 * k, 0.0] for k in range(6)], F)
    sc = scenes.Scene("mirror_remove", 1.0 / 60.0, 80, {"gravity": (0.0, -9.81, 0.0)},
                      [D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0).desc(), shape.desc()], b)
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, -9.81, 0.0)))
    for _ in range(40):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    o.remove_bodies([3])
    for _ in range(40):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    g = world._g
    assert not H.compare_state(o.get_state(), g.get_state())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    world.close()
