"""Point-to-point joints (Point2PointConstraint, dynamics/constraintsolver/Point2PointConstraint.java).

CPU: the oracle's joints hold their pivots together (a chain hanging from fixed points keeps
every pivot gap at millimetres while it swings), the colouring orders joints sharing a dynamic
body, and joints join islands.  GPU: the CUDA step with joints is bit-identical to the oracle,
closed loop, with one solver part per world (the oracle colours like the GPU), with range parts
(cut manifolds; the oracle is fed the GPU's contact order, joints follow the same colouring in
both) and with batch worlds; the joints' applied impulses agree bit for bit."""
import numpy as np
import pytest

from jbgpu import _abi, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle


def _pivot_gaps(state, joints):
    xf = state["transform"]
    gaps = []
    for j in joints:
        a, b = j["a"], j["b"]
        pa = xf[a, :9].reshape(3, 3) @ np.asarray(j["pivot_a"]) + xf[a, 9:]
        pb = (xf[b, :9].reshape(3, 3) @ np.asarray(j["pivot_b"]) + xf[b, 9:]) if b >= 0 else np.asarray(j["pivot_b"])
        gaps.append(np.linalg.norm(pa - pb))
    return np.asarray(gaps)


def test_oracle_chains_keep_their_pivots_together(oracle_lib):
    sc = scenes.jointed_chains(chains=4, links=5, loose=8, seed=1)
    o = pyoracle.OracleWorld(sc)
    worst = 0.0
    for s in range(240):
        o.step(sc.dt)
        worst = max(worst, _pivot_gaps(o.get_state(), sc.meta["joints"]).max())
    assert worst < 0.02, worst
    st = o.get_state()
    links = st["transform"][1:21, 10]
    assert links.min() > 4.0 and links.max() < 10.0          # hanging below the pins, above the plane
    imp = o.joint_impulses()
    assert len(imp) == 20 and np.all(np.isfinite(imp)) and np.any(imp != 0.0)


def test_oracle_joints_join_islands(oracle_lib):
    """Two boxes far apart, joined by a joint, form one island (their pair set is empty)."""
    sc = scenes.jointed_chains(chains=1, links=2, loose=0, seed=2)
    o = pyoracle.OracleWorld(sc)
    o.step(sc.dt)
    tags = o.get_state()["island_tag"]
    assert tags[1] == tags[2] and tags[1] >= 0


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["world_part", "range_parts", "batched"])
def test_gpu_joints_bit_exact(gpu_lib, oracle_lib, case):
    if case == "batched":
        sc = scenes.jointed_chains(chains=3, links=4, loose=6, seed=3, worlds=3)
    else:
        sc = scenes.jointed_chains(chains=6, links=6, loose=24, seed=4)
    cfg = dict(sc.config)
    if case == "range_parts":
        cfg["solver_parts"] = 5
    g = GpuWorld(sc, config=_abi.default_config(**cfg))
    o = pyoracle.OracleWorld(sc)
    for s in range(200):
        g.step(sc.dt)
        if case == "range_parts":
            o.set_explicit_order(g.solver_order())
        o.step(sc.dt)
        assert o.counters()["status_flags"] == 0, s
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
            assert np.array_equal(o.joint_impulses().view(np.uint32), g.joint_impulses().view(np.uint32)), s
    assert g.counters()["status_flags"] == 0
    assert _pivot_gaps(g.get_state(), sc.meta["joints"]).max() < 0.05
    g.close()


@pytest.mark.gpu
def test_gpu_joint_api_errors(gpu_lib):
    sc = scenes.jointed_chains(chains=1, links=2, loose=0, seed=5)
    g = GpuWorld(sc)
    from jbgpu.lib import JbgpuError
    with pytest.raises(JbgpuError):
        g.add_point2point(1, 1, (0, 0, 0), (0, 0, 0))          # a body joined to itself
    with pytest.raises(JbgpuError):
        g.add_point2point(99, -1, (0, 0, 0), (0, 0, 0))        # no such body
    with pytest.raises(JbgpuError):
        g.set_joint_setting(7, 0.3, 1.0, 0.0)
    assert len(g.joint_impulses()) == 2
    g.close()


@pytest.mark.gpu
def test_mirror_pendulum_reads_like_the_reference(gpu_lib, oracle_lib):
    """The reference's usage through the Python mirror: a plane, a box pinned by
    Point2PointConstraint(rbA, pivotInA) and a second box hanging from it by
    Point2PointConstraint(rbA, rbB, pivotInA, pivotInB); stepSimulation for two seconds.  The
    same world built directly on the oracle ends bit-identical, the pivots stay together and
    the joints report their applied impulses."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    ground = D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0)))
    world.addRigidBody(ground)
    shape = D.BoxShape((0.15, 0.45, 0.15))
    links = []
    for i in range(2):
        info = D.RigidBodyConstructionInfo(1.0, None, shape, shape.calculateLocalInertia(1.0))
        info.startWorldTransform = D.Transform(origin=(0.0, 5.5 - 1.0 * i, 0.0))
        body = D.RigidBody(info)
        world.addRigidBody(body)
        links.append(body)
    links[0].setLinearVelocity((1.5, 0.0, 0.0))
    world.addConstraint(D.Point2PointConstraint(links[0], (0.0, 0.5, 0.0)))
    world.addConstraint(D.Point2PointConstraint(links[0], links[1], (0.0, -0.5, 0.0), (0.0, 0.5, 0.0)))
    for _ in range(120):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    g = world._g
    joints = [{"a": 1, "b": -1, "pivot_a": (0.0, 0.5, 0.0), "pivot_b": tuple(world.getConstraint(0).getPivotInB())},
              {"a": 1, "b": 2, "pivot_a": (0.0, -0.5, 0.0), "pivot_b": (0.0, 0.5, 0.0)}]
    assert _pivot_gaps(g.get_state(), joints).max() < 0.02
    assert world.getConstraint(1).getAppliedImpulse() != 0.0
    # the same world on the oracle
    sc = scenes.jointed_chains(chains=1, links=2, loose=0, seed=0)
    sc.bodies["transform"][1, 9:] = (0.0, 5.5, 0.0)
    sc.bodies["transform"][2, 9:] = (0.0, 4.5, 0.0)
    sc.bodies["linear_velocity"][:] = 0.0
    sc.bodies["linear_velocity"][1] = (1.5, 0.0, 0.0)
    sc.meta["joints"] = joints
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(**dict(sc.config, gravity=(0.0, -9.81, 0.0))))
    for _ in range(120):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    assert not H.compare_state(o.get_state(), g.get_state())
    world.close()


# ---- hinges (dynamics/constraintsolver/HingeConstraint.java) ------------------------------
def _hinge_state(state, joints):
    """Per hinge: pivot gap, 1 - |cos| between the two world hinge axes, the relative angle
    about the hinge (exact atan2 of the reference's getHingeAngle projections)."""
    xf = state["transform"]
    out = []
    for j in joints:
        a, b = j["a"], j["b"]
        fa, fb = np.asarray(j["frame_a"], np.float64), np.asarray(j["frame_b"], np.float64)
        Ra = xf[a, :9].reshape(3, 3).astype(np.float64)
        Rb = xf[b, :9].reshape(3, 3).astype(np.float64) if b >= 0 else np.eye(3)
        ob = xf[b, 9:] if b >= 0 else np.zeros(3)
        A, B = fa[:9].reshape(3, 3), fb[:9].reshape(3, 3)
        gap = 0.0 if j.get("angular_only") else np.linalg.norm(Ra @ fa[9:] + xf[a, 9:] - Rb @ fb[9:] - ob)
        mis = 1.0 - abs((Ra @ A[:, 2]) @ (Rb @ B[:, 2]))
        sw = Rb @ B[:, 1]
        out.append((gap, mis, np.arctan2(sw @ (Ra @ A[:, 0]), sw @ (Ra @ A[:, 1]))))
    return np.asarray(out)


def test_hinge_frames_follow_the_constructors():
    from jbgpu import frames
    eye = np.eye(3, dtype=np.float32)
    fa, fb = frames.hinge_frames_two_bodies(eye, (0, -0.5, 0), (0, 0.5, 0), (0, 0, 1), (0, 0, 1))
    assert np.array_equal(fa[:9].reshape(3, 3), eye) and np.array_equal(fa[9:], [0, -0.5, 0])
    assert np.array_equal(fb[:9].reshape(3, 3), np.diag([1, 1, -1]).astype(np.float32))
    # axis along A's x: the reference picks -z and y for the other two columns
    fa, fb = frames.hinge_frames_two_bodies(eye, (0, 0, 0), (0, 0, 0), (1, 0, 0), (1, 0, 0))
    assert np.array_equal(fa[:9].reshape(3, 3), np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]], np.float32))
    # one body: B's frame sits at the pivot's world position; the rest angle is pi
    t = np.concatenate([eye.reshape(9), [1.0, 2.0, 3.0]]).astype(np.float32)
    fa, fb = frames.hinge_frames_one_body(t, (0, 0.5, 0), (0, 0, 1))
    assert np.array_equal(fb[9:], [1.0, 2.5, 3.0])
    A, B = fa[:9].reshape(3, 3), fb[:9].reshape(3, 3)
    assert abs(abs(np.arctan2(B[:, 1] @ A[:, 0], B[:, 1] @ A[:, 1])) - np.pi) < 1e-6
    # by frame: B's z column negated
    fa, fb = frames.hinge_frames_from_frames(t, np.concatenate([eye.reshape(9), [0, 0, 0]]))
    assert np.array_equal(fb[:9].reshape(3, 3), np.diag([1, 1, -1]).astype(np.float32))
    for f in (fa, fb):
        m = f[:9].reshape(3, 3)
        assert np.allclose(m @ m.T, np.eye(3), atol=1e-6)


def test_oracle_hinges_hold(oracle_lib):
    """Hinged chains keep their pivots and axes together while they swing; the limited inner
    hinges stay near +-0.6 rad; the door's motor brings it to its target speed."""
    sc = scenes.hinged_chains(chains=6, links=5, loose=8, seed=1)
    J = sc.meta["joints"]
    o = pyoracle.OracleWorld(sc)
    a0 = _hinge_state(o.get_state(), J)[:, 2]
    steady = [k for k, j in enumerate(J) if "motor" not in j and not j.get("angular_only")]
    limited = [k for k, j in enumerate(J) if "limit" in j]
    worst = np.zeros(3)
    for s in range(240):
        o.step(sc.dt)
        h = _hinge_state(o.get_state(), J)
        if s >= 20:
            worst = np.maximum(worst, [h[steady, 0].max(), h[steady, 1].max(), np.abs(h[limited, 2] - a0[limited]).max()])
    assert o.counters()["status_flags"] == 0
    assert worst[0] < 0.2 and worst[1] < 0.02, worst
    assert worst[2] < 0.75, worst
    door = 1 + 6 * 5
    assert abs(o.get_state()["angular_velocity"][door, 1] + 2.0) < 1e-3
    assert np.any(o.joint_impulses() != 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["world_part", "range_parts", "batched"])
def test_gpu_hinges_bit_exact(gpu_lib, oracle_lib, case):
    if case == "batched":
        sc = scenes.hinged_chains(chains=3, links=4, loose=6, seed=6, worlds=3)
    else:
        sc = scenes.hinged_chains(chains=6, links=5, loose=16, seed=7)
    cfg = dict(sc.config)
    if case == "range_parts":
        cfg["solver_parts"] = 5
    g = GpuWorld(sc, config=_abi.default_config(**cfg))
    o = pyoracle.OracleWorld(sc)
    for s in range(200):
        g.step(sc.dt)
        if case == "range_parts":
            o.set_explicit_order(g.solver_order())
        o.step(sc.dt)
        assert o.counters()["status_flags"] == 0, s
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
            assert np.array_equal(o.joint_impulses().view(np.uint32), g.joint_impulses().view(np.uint32)), s
    assert g.counters()["status_flags"] == 0
    g.close()


@pytest.mark.gpu
def test_gpu_hinge_api_errors(gpu_lib):
    sc = scenes.hinged_chains(chains=1, links=2, loose=0, seed=8)
    g = GpuWorld(sc)
    from jbgpu.lib import JbgpuError
    p2p = g.add_point2point(1, 2, (0, 0, 0), (0, 0, 0))
    with pytest.raises(JbgpuError):
        g.set_joint_setting(0, 0.3, 1.0, 0.0)                   # a hinge has no ConstraintSetting
    with pytest.raises(JbgpuError):
        g.set_hinge_limit(p2p, -1.0, 1.0)                       # not a hinge
    with pytest.raises(JbgpuError):
        g.add_hinge(1, 1, np.zeros(12), np.zeros(12))          # a body hinged to itself
    g.close()


@pytest.mark.gpu
def test_mirror_hinged_door(gpu_lib, oracle_lib):
    """HingeConstraint through the mirror: a door hinged to the fixed body about its vertical
    edge, driven by enableAngularMotor, and a limited hinge to a second panel; the GPU world
    matches the same world built on the oracle bit for bit, the door turns at the motor's speed
    and the limited panel stays within its limit."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    world.addRigidBody(D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.StaticPlaneShape((0.0, 1.0, 0.0), 0.0))))
    shape = D.BoxShape((0.5, 1.0, 0.05))
    panels = []
    for i in range(2):
        info = D.RigidBodyConstructionInfo(2.0, None, shape, shape.calculateLocalInertia(2.0))
        info.startWorldTransform = D.Transform(origin=(1.1 * i, 1.5, 0.0))
        panels.append(D.RigidBody(info))
        world.addRigidBody(panels[-1])
    door = D.HingeConstraint(panels[0], (-0.5, 0.0, 0.0), (0.0, 1.0, 0.0))
    door.enableAngularMotor(True, -1.0, 5.0)
    flap = D.HingeConstraint(panels[0], panels[1], (0.55, 0.0, 0.0), (-0.55, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0))
    flap.setLimit(-0.3, 0.3)
    world.addConstraint(door)
    world.addConstraint(flap)
    for _ in range(90):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    g = world._g
    assert abs(panels[0].getAngularVelocity()[1] + 1.0) < 0.05
    assert abs(flap.getHingeAngle()) < 0.45
    joints = [{"type": "hinge", "a": 1, "b": -1, "frame_a": door.frameA.as12(), "frame_b": door.frameB.as12(),
               "motor": (True, -1.0, 5.0)},
              {"type": "hinge", "a": 1, "b": 2, "frame_a": flap.frameA.as12(), "frame_b": flap.frameB.as12(),
               "limit": (-0.3, 0.3, 0.9, 0.3, 1.0)}]
    shapes = [dict(scenes.PLANE), {"type": _abi.SHAPE_BOX, "params": (0.5, 1.0, 0.05, 0.0), "points": None}]
    bodies = np.zeros(3, scenes.BODY_DTYPE)
    for k in range(3):
        bodies[k] = scenes._bodies(1)[0]
    bodies["shape"] = (0, 1, 1)
    bodies["mass"] = (0.0, 2.0, 2.0)
    bodies["local_inertia"][1:] = scenes.box_inertia(2.0, (0.5, 1.0, 0.05))
    bodies["transform"][1, 9:] = (0.0, 1.5, 0.0)
    bodies["transform"][2, 9:] = (1.1, 1.5, 0.0)
    sc = scenes.Scene("door", 1.0 / 60.0, 90, {"gravity": (0.0, -9.81, 0.0)}, shapes, bodies, meta={"joints": joints})
    o = pyoracle.OracleWorld(sc)
    for _ in range(90):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    assert not H.compare_state(o.get_state(), g.get_state())
    assert np.array_equal(o.joint_impulses().view(np.uint32), g.joint_impulses().view(np.uint32))
    world.close()


# ---- generic 6-dof joints (dynamics/constraintsolver/Generic6DofConstraint.java) ----------
def _d6_state(state, joints):
    """Per joint: pivot gap, and |relative Euler angles| (x, y, z) of frame B in frame A."""
    xf = state["transform"].astype(np.float64)
    out = []
    for j in joints:
        a, b = j["a"], j["b"]
        fa, fb = np.asarray(j["frame_a"], np.float64), np.asarray(j["frame_b"], np.float64)
        Ra, Rb = xf[a, :9].reshape(3, 3), xf[b, :9].reshape(3, 3)
        gap = np.linalg.norm(Ra @ fa[9:] + xf[a, 9:] - Rb @ fb[9:] - xf[b, 9:])
        R = (Ra @ fa[:9].reshape(3, 3)).T @ (Rb @ fb[:9].reshape(3, 3))
        e = (np.arctan2(-R[1, 2], R[2, 2]), np.arcsin(np.clip(R[0, 2], -1, 1)), np.arctan2(-R[0, 1], R[0, 0]))
        out.append((gap,) + tuple(np.abs(e)))
    return np.asarray(out)


def test_oracle_generic6dof_limits_hold(oracle_lib):
    """Locked linear axes keep the pivots together, a free linear axis moves within its +-0.3
    range, angular limits of +-0.4 hold, locked angular axes stay put."""
    sc = scenes.sixdof_chains(chains=4, links=5, loose=8, seed=1)
    J = sc.meta["joints"]
    o = pyoracle.OracleWorld(sc)
    worst = np.zeros((len(J), 4))
    for _ in range(240):
        o.step(sc.dt)
        worst = np.maximum(worst, _d6_state(o.get_state(), J))
    assert o.counters()["status_flags"] == 0
    kinds = np.array([(k // 5) % 4 for k in range(len(J))])
    assert worst[kinds != 2, 0].max() < 0.02 and worst[kinds == 2, 0].max() < 0.36
    assert worst[kinds == 0, 1:].max() < 0.45                       # +-0.4 limits
    assert worst[kinds == 1, 2:].max() < 0.03                       # y and z locked


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["world_part", "range_parts", "batched"])
def test_gpu_generic6dof_bit_exact(gpu_lib, oracle_lib, case):
    if case == "batched":
        sc = scenes.sixdof_chains(chains=4, links=3, loose=4, seed=9, worlds=3)
    else:
        sc = scenes.sixdof_chains(chains=8, links=4, loose=16, seed=10)
    cfg = dict(sc.config)
    if case == "range_parts":
        cfg["solver_parts"] = 5
    g = GpuWorld(sc, config=_abi.default_config(**cfg))
    o = pyoracle.OracleWorld(sc)
    for s in range(200):
        g.step(sc.dt)
        if case == "range_parts":
            o.set_explicit_order(g.solver_order())
        o.step(sc.dt)
        assert o.counters()["status_flags"] == 0, s
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    assert g.counters()["status_flags"] == 0
    g.close()


@pytest.mark.gpu
def test_gpu_generic6dof_api_errors(gpu_lib):
    sc = scenes.sixdof_chains(chains=1, links=2, loose=0, seed=11)
    g = GpuWorld(sc)
    from jbgpu.lib import JbgpuError
    with pytest.raises(JbgpuError):
        g.set_6dof_limit(0, 6, 0.0, 1.0)                        # axes 0..5
    with pytest.raises(JbgpuError):
        g.set_6dof_angular_motor(0, 3, True, 1.0, 1.0)          # angular axes 0..2
    with pytest.raises(JbgpuError):
        g.set_hinge_limit(0, -1.0, 1.0)                          # a 6-dof joint is not a hinge
    p2p = g.add_point2point(2, -1, (0, 0, 0), (0, 0, 0))
    with pytest.raises(JbgpuError):
        g.set_6dof_limit(p2p, 0, 0.0, 1.0)
    g.close()


@pytest.mark.gpu
def test_mirror_generic6dof(gpu_lib):
    """Generic6DofConstraint through the mirror: a box hung from a static anchor, linear axes
    locked, rotation limited to +-0.3 rad about x and locked about y and z, then a motor about x
    switched on between steps through getRotationalLimitMotor."""
    from jbgpu import dynamics as D
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    anchor = D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, D.BoxShape((0.2, 0.2, 0.2))))
    anchor.info.startWorldTransform = D.Transform(origin=(0.0, 5.0, 0.0))
    world.addRigidBody(anchor)
    shape = D.BoxShape((0.15, 0.45, 0.15))
    info = D.RigidBodyConstructionInfo(1.0, None, shape, shape.calculateLocalInertia(1.0))
    info.startWorldTransform = D.Transform(origin=(0.0, 4.3, 0.0))
    box = D.RigidBody(info)
    box.setLinearVelocity((0.0, 0.0, 2.0))
    world.addRigidBody(box)
    c = D.Generic6DofConstraint(box, anchor, D.Transform(origin=(0.0, 0.5, 0.0)), D.Transform(origin=(0.0, -0.2, 0.0)), True)
    c.setAngularLowerLimit((-0.3, 0.0, 0.0))
    c.setAngularUpperLimit((0.3, 0.0, 0.0))
    world.addConstraint(c)
    for _ in range(120):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    st = world._g.get_state()
    j = {"a": 1, "b": 0, "frame_a": c.frameInA.as12(), "frame_b": c.frameInB.as12()}
    gap, ex, ey, ez = _d6_state(st, [j])[0]
    assert gap < 0.02 and ex < 0.4 and ey < 0.02 and ez < 0.02, (gap, ex, ey, ez)
    m = c.getRotationalLimitMotor(0)
    m.enableMotor, m.targetVelocity, m.maxMotorForce = True, 0.5, 50.0
    c.setAngularLowerLimit((1.0, 0.0, 0.0))        # x free (lo > hi)
    c.setAngularUpperLimit((-1.0, 0.0, 0.0))
    for _ in range(60):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    w = box.getAngularVelocity()
    assert abs(abs(w[0]) - 0.5) < 0.05, w
    world.close()


# ---- cone-twist joints (dynamics/constraintsolver/ConeTwistConstraint.java) -----------------
def test_oracle_cone_twist_holds(oracle_lib):
    """Cone-twist chains keep their pivots together and their swing within the cones."""
    sc = scenes.cone_chains(chains=6, links=5, loose=8, seed=1)
    J = sc.meta["joints"]
    o = pyoracle.OracleWorld(sc)
    worst_gap, worst_swing = 0.0, np.zeros(len(J))
    for _ in range(240):
        o.step(sc.dt)
        xf = o.get_state()["transform"].astype(np.float64)
        for k, j in enumerate(J):
            fa, fb = np.asarray(j["frame_a"], np.float64), np.asarray(j["frame_b"], np.float64)
            Ra, Rb = xf[j["a"], :9].reshape(3, 3), xf[j["b"], :9].reshape(3, 3)
            if not j.get("angular_only"):
                worst_gap = max(worst_gap, np.linalg.norm(Ra @ fa[9:] + xf[j["a"], 9:] - Rb @ fb[9:] - xf[j["b"], 9:]))
            A, B = Ra @ fa[:9].reshape(3, 3), Rb @ fb[:9].reshape(3, 3)
            worst_swing[k] = max(worst_swing[k], np.arccos(np.clip(A[:, 0] @ B[:, 0], -1, 1)))
    assert o.counters()["status_flags"] == 0
    assert worst_gap < 0.02, worst_gap
    limited = [k for k, j in enumerate(J) if "limit" in j and not j.get("angular_only")]
    assert worst_swing[limited].max() < 0.7


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["world_part", "range_parts", "batched"])
def test_gpu_cone_twist_bit_exact(gpu_lib, oracle_lib, case):
    if case == "batched":
        sc = scenes.cone_chains(chains=3, links=4, loose=4, seed=12, worlds=3)
    else:
        sc = scenes.cone_chains(chains=6, links=5, loose=8, seed=13)
    cfg = dict(sc.config)
    if case == "range_parts":
        cfg["solver_parts"] = 5
    g = GpuWorld(sc, config=_abi.default_config(**cfg))
    o = pyoracle.OracleWorld(sc)
    for s in range(200):
        g.step(sc.dt)
        if case == "range_parts":
            o.set_explicit_order(g.solver_order())
        o.step(sc.dt)
        assert o.counters()["status_flags"] == 0, s
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
            assert np.array_equal(o.joint_impulses().view(np.uint32), g.joint_impulses().view(np.uint32)), s
    assert g.counters()["status_flags"] == 0
    g.close()


# ---- slider joints (dynamics/constraintsolver/SliderConstraint.java) ------------------------
def test_oracle_slider_rigs(oracle_lib):
    """Limited sliders stop at their limits, the powered one is driven to its limit and spun
    about the axis by its angular motor, the vertical free one slides down to the plane; every
    box stays on its rail's axis."""
    sc = scenes.slider_rigs(rigs=6, loose=8, seed=1)
    J = sc.meta["joints"]
    o = pyoracle.OracleWorld(sc)
    for _ in range(240):
        o.step(sc.dt)
    assert o.counters()["status_flags"] == 0
    st = o.get_state()
    xf = st["transform"]
    for r, j in enumerate(J):
        box, rail = (j["b"], j["a"]) if j["use_a"] else (j["a"], j["b"])
        if r % 3 == 2:
            assert abs(xf[box, 9] - (xf[rail, 9] - 0.5)) < 0.02 and xf[box, 10] < 0.35     # on the plane
        else:
            off = xf[box, 9] - xf[rail, 9]
            assert abs(xf[box, 10] - 3.0) < 0.02 and abs(xf[box, 11] - xf[rail, 11]) < 0.02
            assert abs(abs(off) - (1.0 if r % 3 == 0 else 1.5)) < 0.03, off
    assert abs(abs(st["angular_velocity"][J[1]["b"], 0]) - 2.0) < 0.05


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["world_part", "range_parts", "batched"])
def test_gpu_slider_bit_exact(gpu_lib, oracle_lib, case):
    if case == "batched":
        sc = scenes.slider_rigs(rigs=6, loose=4, seed=14, worlds=3)
    else:
        sc = scenes.slider_rigs(rigs=9, loose=8, seed=15)
    cfg = dict(sc.config)
    if case == "range_parts":
        cfg["solver_parts"] = 5
    g = GpuWorld(sc, config=_abi.default_config(**cfg))
    o = pyoracle.OracleWorld(sc)
    for s in range(200):
        g.step(sc.dt)
        if case == "range_parts":
            o.set_explicit_order(g.solver_order())
        o.step(sc.dt)
        assert o.counters()["status_flags"] == 0, s
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    assert g.counters()["status_flags"] == 0
    g.close()


@pytest.mark.gpu
def test_gpu_slider_params_roundtrip(gpu_lib):
    sc = scenes.slider_rigs(rigs=1, loose=0, seed=16)
    g = GpuWorld(sc)
    p = g.slider_params(0)
    assert p[0] == -1.0 and p[1] == 1.0 and p[5] == np.float32(0.7)
    p[24] = 9.0
    g.set_slider_params(0, p)
    assert g.slider_params(0)[24] == 9.0
    from jbgpu.lib import JbgpuError
    with pytest.raises(JbgpuError):
        g.set_6dof_limit(0, 0, 0.0, 1.0)                        # a slider is not a 6-dof joint
    g.close()
