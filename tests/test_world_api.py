"""The rest of the world and body API a JBullet caller uses between steps:
RigidBody.setDamping / setSleepingThresholds and CollisionObject.setFriction / setRestitution after
the bodies were added (RigidBody.java:224-227, 371-374; CollisionObject.java:186-196),
DynamicsWorld.setInternalTickCallback (DynamicsWorld.java:141-144, DiscreteDynamicsWorld.java:393-395)
and DiscreteDynamicsWorld.removeConstraint (DiscreteDynamicsWorld.java:524-528): the library against
the oracle, closed loop, and through the mirror."""
import numpy as np
import pytest

from jbgpu import _abi, lib as jl, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

F = np.float32


def _assert_same(o, g, where):
    bs = H.compare_state(o.get_state(), g.get_state())
    bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    assert not bs and not bm, (where, bs, bm)


def test_oracle_tick_callback_runs_per_substep(oracle_lib):
    sc = scenes.small_mixed(30, seed=1)
    o = pyoracle.OracleWorld(sc)
    seen = []
    o.set_internal_tick_callback(lambda w, dt: seen.append((w is o, np.float32(dt))))
    n = o.step_simulation(2.5 / 60.0, 4, 1.0 / 60.0)   # localTime starts at 1/60: three substeps
    assert n == 3 and seen == [(True, F(1.0 / 60.0))] * 3
    o.step(1.0 / 30.0, 2)
    assert len(seen) == 5 and seen[-1] == (True, F(1.0 / 30.0))

    def boom(w, dt):
        raise KeyError("from the callback")
    o.set_internal_tick_callback(boom)
    with pytest.raises(KeyError):
        o.step(1.0 / 60.0)
    o.set_internal_tick_callback(None)
    o.step(1.0 / 60.0)


def test_oracle_damping_is_clamped_and_stops_a_body(oracle_lib):
    """setDamping clamps to [0, 1]: linear and angular damping of 5 act as 1 and leave a body
    without gravity or forces still after predictUnconstraintMotion (applyDamping: v *= (1 - 1)^dt)."""
    sc = scenes.small_mixed(20, seed=2)
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, 0.0, 0.0)))
    b = int(np.flatnonzero(sc.bodies["mass"] > 0)[0])
    st = o.get_state()
    st["linear_velocity"][b] = (1.0, 2.0, 3.0)
    st["angular_velocity"][b] = (0.5, 0.0, 0.0)
    o.set_state({"linear_velocity": st["linear_velocity"], "angular_velocity": st["angular_velocity"]})
    o.set_body_properties([b], linear_damping=5.0, angular_damping=5.0)
    o.stage(_abi.STAGE_PREDICT, sc.dt)
    st = o.get_state()
    assert not np.any(st["linear_velocity"][b]) and not np.any(st["angular_velocity"][b])
    with pytest.raises(ValueError):
        o.set_body_properties([b, b], friction=0.1)
    with pytest.raises(ValueError):
        o.remove_joint(0)          # the scene has no joints


@pytest.mark.gpu
def test_body_properties_closed_loop_bit_exact(gpu_lib, oracle_lib):
    sc = scenes.small_mixed(60, seed=8)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    n = len(sc.bodies)
    rng = np.random.default_rng(8)
    for s in range(sc.steps):
        if s in (15, 60, 120):
            idx = rng.choice(np.arange(n), size=20, replace=False).astype(np.int32)
            props = dict(linear_damping=rng.uniform(-0.2, 1.2, 10), angular_damping=rng.uniform(0.0, 0.9, 10),
                         friction=rng.uniform(0.0, 1.5, 10), restitution=rng.uniform(0.0, 0.8, 10),
                         linear_sleeping_threshold=rng.uniform(0.2, 2.0, 10),
                         angular_sleeping_threshold=rng.uniform(0.2, 2.0, 10))
            for w in (o, g):
                w.set_body_properties(idx[:10], **props)
                w.set_body_properties(idx[10:], friction=F(0.05), restitution=None)   # a scalar, a skipped one
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9 or s in (15, 16, 60, 61, 120, 121):
            _assert_same(o, g, s)
    for bad in ([n], [-1], [2, 2]):
        with pytest.raises(jl.JbgpuError):
            g.set_body_properties(bad, friction=0.3)
    g.close()


@pytest.mark.gpu
def test_tick_callback_closed_loop_bit_exact(gpu_lib, oracle_lib):
    """The callback kicks a few bodies and changes one body's gravity after chosen substeps of
    stepSimulation calls that run zero to three substeps; it may not step the world itself."""
    sc = scenes.small_mixed(60, seed=9)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    n = len(sc.bodies)
    ticks = {id(o): [], id(g): []}
    refused = []

    def make(world):
        def cb(w, dt):
            assert w is world
            k = len(ticks[id(w)])
            ticks[id(w)].append(np.float32(dt))
            if k % 3 == 1:
                b = np.array([(7 * k) % n, (7 * k + 3) % n], np.int32)
                w.apply_impulses(b, impulses=[(0.0, 2.0, 0.3), (-1.0, 0.5, 0.0)], torque_impulses=[(0.0, 0.1, 0.0)] * 2)
            if k == 10:
                w.set_body_gravity([5], (0.0, 3.0, 0.0))
            if k == 11 and isinstance(w, GpuWorld):
                try:
                    w.step(dt)
                except jl.JbgpuError:
                    refused.append(k)
        return cb
    o.set_internal_tick_callback(make(o))
    g.set_internal_tick_callback(make(g))
    for s in range(90):
        ts = (1.0 / 60.0) * (0.5, 1.0, 2.2, 3.4)[s % 4]
        no = o.step_simulation(ts, 3, 1.0 / 60.0)
        ng = g.step_simulation(ts, 3, 1.0 / 60.0)
        assert no == ng
        if s % 5 == 4:
            _assert_same(o, g, s)
    assert ticks[id(o)] == ticks[id(g)] and len(ticks[id(g)]) > 60
    assert refused == [11]
    g.set_internal_tick_callback(None)
    o.set_internal_tick_callback(None)
    for _ in range(5):
        o.step(sc.dt)
        g.step(sc.dt)
    assert len(ticks[id(g)]) == len(ticks[id(o)])
    _assert_same(o, g, "after the callback was removed")
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("make", ["jointed", "sixdof"])
def test_remove_joint_closed_loop_bit_exact(gpu_lib, oracle_lib, make):
    sc = (scenes.jointed_chains(chains=4, links=5, loose=8, seed=11) if make == "jointed"
          else scenes.sixdof_chains(chains=4, links=4, loose=6, seed=12))
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    nj = len(g.joint_impulses())
    assert nj >= 12
    removals = {30: [0], 70: [nj // 2, nj // 2], 110: [nj - 3 - 1]}   # first, middle twice, near the end
    for s in range(160):
        for jid in removals.get(s, []):
            for w in (o, g):
                w.remove_joint(jid)
            assert np.array_equal(o.joint_impulses().view(np.uint32), g.joint_impulses().view(np.uint32)), s
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9 or s in (30, 31, 70, 71, 110, 111):
            _assert_same(o, g, s)
            assert np.array_equal(o.joint_impulses().view(np.uint32), g.joint_impulses().view(np.uint32)), s
    assert len(g.joint_impulses()) == nj - 4
    with pytest.raises(jl.JbgpuError):
        g.remove_joint(nj - 4)
    g.close()


@pytest.mark.gpu
def test_mirror_world_api_reads_like_the_reference(gpu_lib, oracle_lib):
    """Through the mirror: a pendulum whose constraint is removed, forces and torques applied
    between steps and from a tick callback, damping and friction changed after addRigidBody,
    clearForces; the same sequence on the oracle ends bit-identical."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0))))
    box = D.BoxShape((0.3, 0.3, 0.3))
    bodies = []
    for k in range(3):
        info = D.RigidBodyConstructionInfo(1.0, None, box, box.calculateLocalInertia(1.0))
        info.startWorldTransform = D.Transform(origin=(1.5 * k, 2.0 + k, 0.0))
        b = D.RigidBody(info)
        world.addRigidBody(b)
        bodies.append(b)
    p2p = D.Point2PointConstraint(bodies[2], (0.0, 0.5, 0.0))
    world.addConstraint(p2p)
    calls = []

    class Tick:
        def internalTick(self, w, dt):
            calls.append(dt)
            if len(calls) % 2 == 0:
                bodies[0].applyCentralForce((3.0, 0.0, 0.0))

    world.setInternalTickCallback(Tick(), "info")
    assert world.getWorldUserInfo() == "info"
    for _ in range(20):
        world.stepSimulation(1.0 / 30.0, 2, 1.0 / 60.0)
    bodies[1].setDamping(0.3, 2.0)                 # angular damping clamps to 1
    bodies[1].setFriction(0.9)
    bodies[0].applyForce((0.0, 5.0, 0.0), (0.1, 0.0, 0.2))
    bodies[0].applyTorque((0.0, 0.0, 0.4))
    bodies[1].applyCentralForce((1.0, 1.0, 1.0))
    bodies[1].clearForces()
    hung = float(bodies[2].getCenterOfMassPosition()[1])
    world.removeConstraint(p2p)
    assert world.getNumConstraints() == 0
    for _ in range(20):
        world.stepSimulation(1.0 / 30.0, 2, 1.0 / 60.0)
    assert bodies[1].getAngularDamping() == 1.0 and bodies[1].getFriction() == 0.9
    assert bodies[2].getCenterOfMassPosition()[1] < hung - 1.0     # freed from its pivot, it fell

    b = scenes._bodies(4)
    b["shape"] = [0, 1, 1, 1]
    b["mass"] = [0.0, 1.0, 1.0, 1.0]
    b["local_inertia"][1:] = box.calculateLocalInertia(1.0)
    b["transform"][:, [0, 4, 8]] = 1.0
    b["transform"][1:, 9:] = np.array([[0, 2, 0], [1.5, 3, 0], [3, 4, 0]], F)
    sc = scenes.Scene("mirror_world_api", 1.0 / 60.0, 80, {"gravity": (0.0, -9.81, 0.0)},
                      [D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0).desc(), box.desc()], b)
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, -9.81, 0.0)))
    pivot_b = np.array([3.0, 4.5, 0.0], F)                           # rbA's transform applied to pivotInA
    o.add_point2point(3, -1, (0.0, 0.5, 0.0), pivot_b)
    n_ticks = [0]

    def force(w, body, f=None, t=None):
        st = w.get_state()
        if f is not None:
            st["total_force"][body] += np.asarray(f, F)
        if t is not None:
            st["total_torque"][body] += np.asarray(t, F)
        w.set_state({"total_force": st["total_force"], "total_torque": st["total_torque"]})

    def tick(w, dt):
        n_ticks[0] += 1
        if n_ticks[0] % 2 == 0:
            force(w, 1, f=(3.0, 0.0, 0.0))
    o.set_internal_tick_callback(tick)
    for _ in range(20):
        o.step_simulation(1.0 / 30.0, 2, 1.0 / 60.0)
    o.set_body_properties([2], linear_damping=0.3, angular_damping=1.0, friction=0.9)
    force(o, 1, f=(0.0, 5.0, 0.0), t=D._crs((0.1, 0.0, 0.2), (0.0, 5.0, 0.0)) + np.array([0.0, 0.0, 0.4], F))
    o.remove_joint(0)
    for _ in range(20):
        o.step_simulation(1.0 / 30.0, 2, 1.0 / 60.0)
    assert n_ticks[0] == len(calls)
    g = world._g
    assert not H.compare_state(o.get_state(), g.get_state())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    world.close()


def test_mirror_getters_without_a_device():
    """Getters that need no device state: clamped damping, flags, inverse local inertia, the
    orientation of a basis (libGDX Quaternion.setFromMatrix), the velocity at a point."""
    from jbgpu import dynamics as D
    box = D.BoxShape((0.5, 0.25, 0.1))
    info = D.RigidBodyConstructionInfo(2.0, None, box, box.calculateLocalInertia(2.0))
    b = D.RigidBody(info)
    b.setDamping(-1.0, 0.25)
    assert b.getLinearDamping() == 0.0 and b.getAngularDamping() == 0.25
    assert not b.isStaticObject() and b.hasContactResponse() and b.mergesSimulationIslands()
    assert np.allclose(b.getInvInertiaDiagLocal() * np.asarray(info.localInertia, F), 1.0)
    c, s = F(np.cos(0.3)), F(np.sin(0.3))
    q = D._quat_from_basis(np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], F))
    assert np.allclose(q, [0.0, 0.0, np.sin(0.15), np.cos(0.15)], atol=1e-6)
    q = D._quat_from_basis(np.diag([F(-1.0), F(-1.0), F(1.0)]))        # trace < 0: a diagonal branch
    assert np.allclose(np.abs(q), [0.0, 0.0, 1.0, 0.0])
    assert np.array_equal(D._crs((1, 0, 0), (0, 1, 0)), np.array([0, 0, 1], F))
    static = D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0)))
    assert static.isStaticObject() and static.isStaticOrKinematicObject() and not static.mergesSimulationIslands()


@pytest.mark.gpu
def test_mirror_collision_detection_without_a_step(gpu_lib, oracle_lib):
    """performDiscreteCollisionDetection after a body was moved by hand: the pairs and manifolds
    equal the oracle's aabb, pair and narrowphase stages on the same state, and no body moved."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0))))
    box = D.BoxShape((0.5, 0.5, 0.5))
    bodies = []
    for k in range(3):
        info = D.RigidBodyConstructionInfo(1.0, None, box, box.calculateLocalInertia(1.0))
        info.startWorldTransform = D.Transform(origin=(2.0 * k, 0.6, 0.0))
        bodies.append(D.RigidBody(info))
        world.addRigidBody(bodies[-1])
    for _ in range(10):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    before = world._g.get_state()["transform"].copy()
    bodies[2].setWorldTransform(D.Transform(origin=(0.6, 1.5, 0.1)))   # onto body 1
    world.performDiscreteCollisionDetection()
    assert world.getDispatcher().getNumManifolds() >= 3
    g = world._g

    b = scenes._bodies(4)
    b["shape"] = [0, 1, 1, 1]
    b["mass"] = [0.0, 1.0, 1.0, 1.0]
    b["local_inertia"][1:] = box.calculateLocalInertia(1.0)
    b["transform"][:, [0, 4, 8]] = 1.0
    b["transform"][1:, 9:] = np.array([[0, 0.6, 0], [2, 0.6, 0], [4, 0.6, 0]], F)
    sc = scenes.Scene("mirror_collide", 1.0 / 60.0, 10, {"gravity": (0.0, -9.81, 0.0)},
                      [D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0).desc(), box.desc()], b)
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, -9.81, 0.0)))
    for _ in range(10):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    t = o.get_state()["transform"]
    t[3] = D.Transform(origin=(0.6, 1.5, 0.1)).as12()
    o.set_state({"transform": t})
    for st in (_abi.STAGE_AABB, _abi.STAGE_PAIRS, _abi.STAGE_NARROWPHASE):
        o.stage(st, 1.0 / 60.0)
    assert not H.compare_state(o.get_state(), g.get_state())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    after = g.get_state()["transform"]
    assert np.array_equal(np.delete(after, 3, 0), np.delete(before, 3, 0))
    world.close()


def _interp(o, g, where):
    a, b = o.get_interpolated_transforms(), g.get_interpolated_transforms()
    assert a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32)), where


@pytest.mark.gpu
@pytest.mark.parametrize("make", ["mixed", "ccd"])
def test_interpolated_transforms_bit_exact(gpu_lib, oracle_lib, make):
    """synchronizeMotionStates' transforms with a residual localTime (time steps that are not
    multiples of the fixed step), sleeping bodies and, in the CCD scene, clamped bodies
    (hitFraction 0)."""
    sc = scenes.small_mixed(60, seed=13) if make == "mixed" else scenes.ccd_shots(seed=4)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    _interp(o, g, "start")
    for s in range(120):
        ts = (1.0 / 60.0) * (0.37, 1.0, 1.61, 2.9)[s % 4]
        assert o.step_simulation(ts, 2, 1.0 / 60.0) == g.step_simulation(ts, 2, 1.0 / 60.0)
        if s % 3 == 0:
            _interp(o, g, s)
            assert not H.compare_state(o.get_state(), g.get_state()), s
    g.close()


@pytest.mark.gpu
def test_mirror_motion_states_read_like_the_reference(gpu_lib, oracle_lib):
    """A dynamic body with a MotionState gets setWorldTransform after every stepSimulation call,
    with the oracle's interpolated transform; a static body's motion state is left alone."""
    from jbgpu import dynamics as D

    class Motion:
        def __init__(self):
            self.calls = 0
            self.t = None

        def setWorldTransform(self, t):
            self.calls += 1
            self.t = t.as12()

    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    ground_motion = Motion()
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, ground_motion,
                                                               D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0))))
    sph = D.SphereShape(0.5)
    motion = Motion()
    info = D.RigidBodyConstructionInfo(1.0, motion, sph, sph.calculateLocalInertia(1.0))
    info.startWorldTransform = D.Transform(origin=(0.0, 3.0, 0.0))
    ball = D.RigidBody(info)
    world.addRigidBody(ball)
    ball.setAngularVelocity((0.0, 2.0, 1.0))
    b = scenes._bodies(2)
    b["shape"] = [0, 1]
    b["mass"] = [0.0, 1.0]
    b["local_inertia"][1] = sph.calculateLocalInertia(1.0)
    b["transform"][:, [0, 4, 8]] = 1.0
    b["transform"][1, 9:] = (0.0, 3.0, 0.0)
    b["angular_velocity"][1] = (0.0, 2.0, 1.0)
    sc = scenes.Scene("mirror_motion", 1.0 / 60.0, 40, {"gravity": (0.0, -9.81, 0.0)},
                      [D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0).desc(), sph.desc()], b)
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, -9.81, 0.0)))
    for s in range(40):
        ts = (1.0 / 60.0) * (0.5 if s % 2 else 1.3)
        world.stepSimulation(ts, 2, 1.0 / 60.0)
        o.step_simulation(ts, 2, 1.0 / 60.0)
        want = o.get_interpolated_transforms()[1]
        assert np.array_equal(motion.t.view(np.uint32), want.view(np.uint32)), s
    assert motion.calls == 40 and ground_motion.calls == 0
    world.close()


@pytest.mark.gpu
def test_tick_callback_removes_bodies_between_substeps(gpu_lib, oracle_lib):
    """Bodies removed from inside the tick callback are gone from the next substep on, in the
    same stepSimulation call; the worlds stay bit-identical."""
    sc = scenes.small_mixed(60, seed=14)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    removals = {4: [10, 20], 9: [3], 15: [len(sc.bodies) - 5]}

    def make():
        count = [0]

        def cb(w, dt):
            k = count[0]
            count[0] += 1
            if k in removals:
                w.remove_bodies(removals[k])
        return cb, count
    cbo, co = make()
    cbg, cg = make()
    o.set_internal_tick_callback(cbo)
    g.set_internal_tick_callback(cbg)
    for s in range(40):
        ts = (1.0 / 60.0) * (2.5 if s % 2 else 1.0)      # one or two substeps per call
        assert o.step_simulation(ts, 3, 1.0 / 60.0) == g.step_simulation(ts, 3, 1.0 / 60.0)
        _assert_same(o, g, s)
    assert co[0] == cg[0] > 16
    assert len(g.get_state()["transform"]) == len(sc.bodies) - 4
    g.close()
