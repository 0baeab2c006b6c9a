"""Kinematic and trigger bodies: CollisionFlags.KINEMATIC_OBJECT with saveKinematicState
(DiscreteDynamicsWorld.java:105-119, RigidBody.java:190-205) and NO_CONTACT_RESPONSE
(CollisionDispatcher.needsResponse), with the activation state a body is given before it is added.

CPU: the oracle's kinematic velocities are TransformUtil.calculateVelocity of the caller's pose
change, trigger bodies are passed through, an unmoved kinematic body with the default activation
falls asleep, and the body descriptor checks its flags.  GPU: the library against the oracle, closed
loop and stage by stage (the saveKinematicState stage included), and through the mirror's
setCollisionFlags / setActivationState / motion-state path."""
import ctypes as C

import numpy as np
import pytest

from jbgpu import _abi, lib as jl, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

F = np.float32


def _drive(worlds, sc, step):
    """The platforms' poses at `step` written into every world (the caller moving them)."""
    idx = sc.meta["kinematic"]["bodies"]
    pose = scenes.kinematic_pose(sc, step)
    for w in worlds:
        t = w.get_state()["transform"]
        t[idx] = pose
        w.set_state({"transform": t})


def _velocity(t0, t1, dt):
    """TransformUtil.calculateVelocity's linear part in binary32."""
    return ((t1[9:] - t0[9:]) * F(F(1.0) / F(dt))).astype(F)


def test_oracle_kinematic_velocities_triggers_and_sleep(oracle_lib):
    sc = scenes.kinematic_platforms(seed=3)
    o = pyoracle.OracleWorld(sc)
    idx = sc.meta["kinematic"]["bodies"]
    prev = sc.bodies["transform"][idx].copy()
    for s in range(sc.steps):
        _drive([o], sc, s + 1)
        o.step(sc.dt)
        if s in (0, 57, 200):
            st = o.get_state()
            cur = scenes.kinematic_pose(sc, s + 1)
            for j, b in enumerate(idx):
                assert np.array_equal(st["linear_velocity"][b], _velocity(prev[j], cur[j], sc.dt))
        prev = scenes.kinematic_pose(sc, s + 1)
    st = o.get_state()
    n = len(sc.bodies)
    trig_box, dropped, trig_sphere, resting = n - 4, n - 3, n - 2, n - 1
    assert st["transform"][dropped, 10] < F(0.35)        # fell through the trigger box to the ground
    assert st["transform"][trig_sphere, 10] < F(-10.0)   # fell through the ground
    assert st["activation_state"][resting] == _abi.ISLAND_SLEEPING
    assert np.all(st["activation_state"][idx] == _abi.DISABLE_DEACTIVATION)
    assert st["transform"][trig_box, 10] == F(0.5)
    assert o.counters()["solver_manifolds"] > 0


def test_body_descriptor_layout(gpu_lib):
    assert C.sizeof(_abi.BodyDesc) == scenes.BODY_DTYPE.itemsize
    assert scenes.BODY_DTYPE.names[-2:] == ("collision_flags", "activation_state")


@pytest.mark.gpu
def test_unsupported_body_flags_are_rejected(gpu_lib):
    for field, value in (("collision_flags", 8), ("activation_state", 6)):
        sc = scenes.kinematic_platforms(seed=1)
        sc.bodies[field][3] = value
        with pytest.raises(jl.JbgpuError):
            GpuWorld(sc)


@pytest.mark.gpu
def test_kinematic_and_trigger_closed_loop_bit_exact(gpu_lib, oracle_lib):
    sc = scenes.kinematic_platforms(seed=3)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    for s in range(sc.steps):
        _drive([o, g], sc, s + 1)
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    co, cg = o.counters(), g.counters()
    for k in ("pairs", "manifolds", "contacts", "solver_manifolds", "solver_rows"):
        assert co[k] == cg[k], (k, co[k], cg[k])
    assert cg["status_flags"] == 0 and cg["solver_manifolds"] > 0
    g.close()


@pytest.mark.gpu
def test_step_simulation_saves_kinematic_state_once_per_call(gpu_lib, oracle_lib):
    """stepSimulation saves the kinematic state once per call, with the fixed time step, and not
    at all when the call runs no substep."""
    sc = scenes.kinematic_platforms(seed=5, steps=90)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    for s in range(sc.steps):
        _drive([o, g], sc, s + 1)
        ts = (1.0 / 60.0) * (0.5 if s % 3 == 0 else 1.5)   # some calls run no substep, some two
        no = o.step_simulation(ts, 2, 1.0 / 60.0)
        ng = g.step_simulation(ts, 2, 1.0 / 60.0)
        assert no == ng
        bs = H.compare_state(o.get_state(), g.get_state())
        assert not bs, (s, bs)
    g.close()


STAGES = [_abi.STAGE_SAVE_KINEMATIC, _abi.STAGE_APPLY_GRAVITY, _abi.STAGE_PREDICT, _abi.STAGE_AABB, _abi.STAGE_PAIRS,
          _abi.STAGE_NARROWPHASE, _abi.STAGE_ISLANDS, _abi.STAGE_SOLVE, _abi.STAGE_INTEGRATE, _abi.STAGE_ACTIVATION]


@pytest.mark.gpu
@pytest.mark.parametrize("warm", [0, 50, 150])
def test_kinematic_stage_by_stage_bit_exact(gpu_lib, oracle_lib, warm):
    sc = scenes.kinematic_platforms(seed=7)
    ref = pyoracle.OracleWorld(sc)
    for s in range(warm):
        _drive([ref], sc, s + 1)
        ref.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    H.copy_world(ref, o)
    H.copy_world(ref, g)
    _drive([o, g], sc, warm + 1)
    for st in STAGES:
        H.copy_world(o, g)
        o.stage(st, sc.dt)
        g.stage(st, sc.dt)
        bs = H.compare_state(o.get_state(), g.get_state())
        bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
        assert not bs and not bm, (st, bs, bm)
    g.close()


@pytest.mark.gpu
def test_mirror_kinematic_platform_reads_like_the_reference(gpu_lib, oracle_lib):
    """The reference's usage through the mirror: a kinematic platform (setCollisionFlags,
    setActivationState(DISABLE_DEACTIVATION)) driven through its motion state, a box on it and a
    trigger sphere; the same world on the oracle, the platform moved by the caller, ends
    bit-identical."""
    from jbgpu import dynamics as D

    class Motion:
        def __init__(self, t):
            self.t = t

        def getWorldTransform(self):
            return self.t

    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    ground = D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0)))
    world.addRigidBody(ground)
    plat_shape = D.BoxShape((1.5, 0.2, 1.5))
    motion = Motion(D.Transform(origin=(0.0, 2.0, 0.0)))
    info = D.RigidBodyConstructionInfo(0.0, motion, plat_shape)
    info.startWorldTransform = D.Transform(origin=(0.0, 2.0, 0.0))
    plat = D.RigidBody(info)
    plat.setCollisionFlags(plat.getCollisionFlags() | _abi.CF_KINEMATIC_OBJECT)
    plat.setActivationState(_abi.DISABLE_DEACTIVATION)
    world.addRigidBody(plat)
    box_shape = D.BoxShape((0.3, 0.3, 0.3))
    binfo = D.RigidBodyConstructionInfo(1.0, None, box_shape, box_shape.calculateLocalInertia(1.0))
    binfo.startWorldTransform = D.Transform(origin=(0.2, 2.6, 0.1))
    world.addRigidBody(D.RigidBody(binfo))
    sph = D.SphereShape(0.4)
    sinfo = D.RigidBodyConstructionInfo(2.0, None, sph, sph.calculateLocalInertia(2.0))
    sinfo.startWorldTransform = D.Transform(origin=(4.0, 3.0, 0.0))
    trig = D.RigidBody(sinfo)
    trig.setCollisionFlags(_abi.CF_NO_CONTACT_RESPONSE)
    world.addRigidBody(trig)
    poses = []
    for s in range(120):
        x = np.float32(1.2 * np.sin(0.8 * (s + 1) / 60.0))
        pose = D.Transform(origin=(float(x), 2.0, 0.0))
        motion.t = pose
        poses.append(pose.as12())
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    g = world._g
    assert plat.getCollisionFlags() == _abi.CF_STATIC_OBJECT | _abi.CF_KINEMATIC_OBJECT
    b = scenes._bodies(4)
    b["shape"] = [0, 1, 2, 3]
    b["mass"] = [0.0, 0.0, 1.0, 2.0]
    b["collision_flags"] = [0, _abi.CF_KINEMATIC_OBJECT, 0, _abi.CF_NO_CONTACT_RESPONSE]
    b["activation_state"] = [0, _abi.DISABLE_DEACTIVATION, 0, 0]
    b["local_inertia"][2] = box_shape.calculateLocalInertia(1.0)
    b["local_inertia"][3] = sph.calculateLocalInertia(2.0)
    b["transform"][:, [0, 4, 8]] = 1.0
    b["transform"][:, 9:] = np.array([[0, 0, 0], [0.0, 2.0, 0.0], [0.2, 2.6, 0.1], [4.0, 3.0, 0.0]], F)
    sc = scenes.Scene("mirror_kinematic", 1.0 / 60.0, 120, {"gravity": (0.0, -9.81, 0.0)},
                      [ground.info.collisionShape.desc(), plat_shape.desc(), box_shape.desc(), sph.desc()], b)
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, -9.81, 0.0)))
    for s in range(120):
        t = o.get_state()["transform"]
        t[1] = poses[s]
        o.set_state({"transform": t})
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    assert not H.compare_state(o.get_state(), g.get_state())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    st = g.get_state()
    assert st["transform"][3, 10] < 0.0           # the trigger sphere fell through the ground
    assert abs(float(st["transform"][2, 9]) - float(st["transform"][1, 9])) < 1.0   # the box rides the platform
    world.close()
