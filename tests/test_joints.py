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
