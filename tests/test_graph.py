"""The step replayed as CUDA graphs (jbgpu_world_set_graph; the default, jbgpu_config.step_graphs)
against the same step launched kernel by kernel: body state, manifolds and joint impulses
bit-identical after every checked step, on a falling mix of every shape (the pair count grows, so the pair buffers grow and the graphs are
captured again), on batch worlds with joints, across a change of the iteration count, and with
the graphs actually in use (held, no capture failure)."""
import numpy as np
import pytest

from jbgpu import _abi, scenes
from jbgpu.lib import GpuWorld

import harness as H


def _pair(sc, **cfg):
    c = _abi.default_config(**dict(sc.config, **cfg))
    eager = GpuWorld(sc, config=c)
    eager.set_graph(False)
    graph = GpuWorld(sc, config=c)
    graph.set_graph(True)
    return eager, graph


def _same(a, b, step):
    bs = H.compare_state(a.get_state(), b.get_state())
    bm = H.compare_manifolds(a.get_manifolds(), b.get_manifolds())
    assert not bs and not bm, (step, bs, bm)


@pytest.mark.gpu
@pytest.mark.parametrize("scene", ["small_mixed", "hinged_batched", "boxes"])
def test_graph_step_matches_launches(gpu_lib, scene):
    if scene == "small_mixed":
        sc = scenes.small_mixed(n=200, seed=21)
    elif scene == "hinged_batched":
        sc = scenes.hinged_chains(chains=3, links=4, loose=8, seed=22, worlds=6)
    else:
        sc = scenes.boxes_on_plane(n=1000, seed=23)
    eager, graph = _pair(sc, broadphase_rebuild_interval=3)
    for s in range(150):
        eager.step_simulation(sc.dt, 1, sc.dt)
        graph.step_simulation(sc.dt, 1, sc.dt)
        if s % 25 == 24 or s < 3:
            _same(eager, graph, s)
            if scene == "hinged_batched":
                assert np.array_equal(eager.joint_impulses().view(np.uint32), graph.joint_impulses().view(np.uint32))
    n, err = graph.graph_status()
    assert err == "" and n >= 2, (n, err)
    assert graph.counters()["status_flags"] == 0
    eager.close()
    graph.close()


@pytest.mark.gpu
def test_graph_follows_setting_changes(gpu_lib):
    """Settings baked into captured launches (the iteration count) drop the graphs."""
    sc = scenes.small_mixed(n=120, seed=24)
    eager, graph = _pair(sc)
    for s in range(60):
        if s == 30:
            for w in (eager, graph):
                w.set_solver_iterations(4)
        eager.step(sc.dt)
        graph.step(sc.dt)
    _same(eager, graph, 60)
    assert graph.graph_status()[1] == ""
    eager.close()
    graph.close()
