"""RigidBody.applyCentralImpulse / applyImpulse / applyTorqueImpulse (RigidBody.java:395-427)
between steps: the library against the oracle, closed loop, and through the mirror."""
import numpy as np
import pytest

from jbgpu import lib as jl, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

F = np.float32


def _kicks(n, seed):
    r = np.random.default_rng(seed)
    idx = r.choice(np.arange(n), size=min(24, n), replace=False).astype(np.int32)
    return idx, r.normal(0, 3, (len(idx), 3)).astype(F), r.normal(0, 0.3, (len(idx), 3)).astype(F), \
        r.normal(0, 0.5, (len(idx), 3)).astype(F)


def test_oracle_impulse_velocity_change(oracle_lib):
    """A central impulse changes only the linear velocity, by impulse / mass; a static body (body 0
    of the mixed scene is the ground) is unchanged by applyImpulse."""
    sc = scenes.small_mixed(60, seed=2)
    o = pyoracle.OracleWorld(sc)
    st0 = o.get_state()
    b = int(np.flatnonzero(sc.bodies["mass"] > 0)[0])
    m = F(sc.bodies["mass"][b])
    o.apply_impulses([b], impulses=[(m, 0.0, -m)])
    o.apply_impulses([0], impulses=[(5.0, 5.0, 5.0)], rel_pos=[(1.0, 0.0, 0.0)])
    st = o.get_state()
    assert np.array_equal(st["angular_velocity"], st0["angular_velocity"])
    dv = st["linear_velocity"][b] - st0["linear_velocity"][b]
    assert np.allclose(dv, [1.0, 0.0, -1.0], atol=1e-6), dv
    assert np.array_equal(st["linear_velocity"][0], st0["linear_velocity"][0])
    with pytest.raises(ValueError):
        o.apply_impulses([len(sc.bodies)], impulses=[(1.0, 0.0, 0.0)])


@pytest.mark.gpu
def test_impulses_closed_loop_bit_exact(gpu_lib, oracle_lib):
    sc = scenes.small_mixed(60, seed=6)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    n = len(sc.bodies)
    for s in range(sc.steps):
        if s in (20, 75, 130):
            idx, J, r, T = _kicks(n, 100 + s)
            third = len(idx) // 3
            for w in (o, g):
                w.apply_impulses(idx[:third], impulses=J[:third])                                  # central
                w.apply_impulses(idx[third:2 * third], impulses=J[third:2 * third], rel_pos=r[third:2 * third])
                w.apply_impulses(idx[2 * third:], torque_impulses=T[2 * third:])                   # torque
                w.apply_impulses(idx[:4], impulses=J[:4], rel_pos=r[:4], torque_impulses=T[:4])    # all three
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9 or s in (20, 21, 75, 76, 130, 131):
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    co, cg = o.counters(), g.counters()
    for k in ("pairs", "manifolds", "contacts", "solver_manifolds", "solver_rows"):
        assert co[k] == cg[k], (k, co[k], cg[k])
    for bad in ([n], [-1], [3, 3]):
        with pytest.raises(jl.JbgpuError):
            g.apply_impulses(bad, impulses=[(1.0, 0.0, 0.0)] * len(bad))
    assert not H.compare_state(o.get_state(), g.get_state())   # a refused call changes nothing
    g.close()


@pytest.mark.gpu
def test_mirror_impulses_read_like_the_reference(gpu_lib, oracle_lib):
    """A ball kicked sideways after it settles, a box hit off-centre and spun: the same calls on the
    oracle end bit-identical, and the kicked ball moves the way it was pushed."""
    from jbgpu import _abi
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0))))
    sph = D.SphereShape(0.5)
    box = D.BoxShape((0.4, 0.2, 0.3))
    shapes = [sph, box]
    bodies = []
    for k, sh in enumerate(shapes):
        info = D.RigidBodyConstructionInfo(2.0, None, sh, sh.calculateLocalInertia(2.0))
        info.startWorldTransform = D.Transform(origin=(3.0 * k, 1.0, 0.0))
        b = D.RigidBody(info)
        world.addRigidBody(b)
        bodies.append(b)
    for _ in range(30):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    bodies[0].applyCentralImpulse((4.0, 0.0, 0.0))
    bodies[1].applyImpulse((0.0, 6.0, 0.0), (0.3, 0.0, 0.1))
    bodies[1].applyTorqueImpulse((0.0, 0.2, 0.0))
    for _ in range(30):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    b = scenes._bodies(3)
    b["shape"] = [0, 1, 2]
    b["mass"] = [0.0, 2.0, 2.0]
    b["local_inertia"][1] = sph.calculateLocalInertia(2.0)
    b["local_inertia"][2] = box.calculateLocalInertia(2.0)
    b["transform"][:, [0, 4, 8]] = 1.0
    b["transform"][1:, 9:] = np.array([[0, 1, 0], [3, 1, 0]], F)
    sc = scenes.Scene("mirror_impulses", 1.0 / 60.0, 60, {"gravity": (0.0, -9.81, 0.0)},
                      [D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0).desc(), sph.desc(), box.desc()], b)
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, -9.81, 0.0)))
    for _ in range(30):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    o.apply_impulses([1], impulses=[(4.0, 0.0, 0.0)])
    o.apply_impulses([2], impulses=[(0.0, 6.0, 0.0)], rel_pos=[(0.3, 0.0, 0.1)])
    o.apply_impulses([2], torque_impulses=[(0.0, 0.2, 0.0)])
    for _ in range(30):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    g = world._g
    assert not H.compare_state(o.get_state(), g.get_state())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    assert g.get_state()["transform"][1, 9] > F(0.5)     # the ball rolled the way it was pushed
    with pytest.raises(RuntimeError):
        D.RigidBody(D.RigidBodyConstructionInfo(1.0, None, sph, sph.calculateLocalInertia(1.0))).applyCentralImpulse((1, 0, 0))
    world.close()
