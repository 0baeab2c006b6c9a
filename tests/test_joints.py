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
