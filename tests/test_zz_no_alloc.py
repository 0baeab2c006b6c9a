"""jbgpu_world_narrowphase_static, the narrowphase entry point that allocates nothing: its EPA
pass runs on scratch compiled into the library.  On identical worlds it must give the same
manifolds and counters as the narrowphase stage of jbgpu_world_stage (which uses the world's
own EPA arena), on two calls in a row; and it must reject out-of-range slot counts.

Kept in a file of its own, collected last, so that it also runs after every other test has
used the library in the same process."""
import ctypes as C

import numpy as np
import pytest

from jbgpu import _abi, scenes
from jbgpu._build import LIB
from jbgpu.lib import GpuWorld

import harness as H

pytestmark = pytest.mark.gpu

F = np.float32
STATIC_EPA_SLOTS_MAX = 32      # JBGPU_STATIC_EPA_SLOTS_MAX of include/jbgpu.h


def _entry():
    L = C.CDLL(LIB)
    f = L.jbgpu_world_narrowphase_static
    f.argtypes = [C.c_void_p, C.c_int32]
    f.restype = C.c_int
    L.jbgpu_last_error.argtypes = []
    L.jbgpu_last_error.restype = C.c_char_p
    return f, L


def overlapping_pairs(n_pairs=40, seed=11):
    """Boxes and hulls in pairs whose cores overlap by 0.2-0.4, so that GJK ends in the
    penetration case and every pair goes through EPA; no gravity, no plane."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = rng.standard_normal((24, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    hull = (d * np.array([0.6, 0.45, 0.5])).astype(F)
    shapes = [{"type": _abi.SHAPE_BOX, "params": (0.5, 0.4, 0.45, 0.0), "points": None},
              {"type": _abi.SHAPE_CONVEX_HULL, "params": (0, 0, 0, 0), "points": hull}]
    n = 2 * n_pairs
    b = scenes._bodies(n)
    b["shape"] = np.arange(n) % 2
    b["mass"] = 1.0
    b["local_inertia"][0::2] = scenes.box_inertia(F(1.0), (0.5, 0.4, 0.45))
    b["local_inertia"][1::2] = scenes.hull_inertia(F(1.0), hull)
    R = scenes.random_rotations(rng, n)
    pos = np.zeros((n, 3))
    for k in range(n_pairs):
        c = np.array([(k % 8) * 4.0, 2.0, (k // 8) * 4.0])
        off = rng.standard_normal(3)
        off *= rng.uniform(0.5, 0.7) / np.linalg.norm(off)
        pos[2 * k] = c
        pos[2 * k + 1] = c + off
    scenes._set_transforms(b, R, pos)
    return scenes.Scene("overlapping_pairs", 1.0 / 60.0, 1, {"gravity": (0.0, 0.0, 0.0)}, shapes, b)


def _to_pairs(g, dt):
    for st in (_abi.STAGE_APPLY_GRAVITY, _abi.STAGE_PREDICT, _abi.STAGE_AABB, _abi.STAGE_PAIRS):
        g.stage(st, dt)


def test_static_scratch_matches_the_narrowphase_stage(gpu_lib):
    narrow_static, L = _entry()
    sc = overlapping_pairs()
    ref, mine = GpuWorld(sc), GpuWorld(sc)
    _to_pairs(ref, sc.dt)
    _to_pairs(mine, sc.dt)
    assert np.array_equal(ref.get_pairs(), mine.get_pairs())
    for call, slots in enumerate((7, STATIC_EPA_SLOTS_MAX)):
        ref.stage(_abi.STAGE_NARROWPHASE, sc.dt)
        rc = narrow_static(mine.h, slots)
        assert rc == 0, (call, rc, L.jbgpu_last_error())
        cr, cm = ref.counters(), mine.counters()
        assert cr["epa_calls"] >= 30, cr          # the scene exercises EPA, more pairs than slots
        for k in ("gjk_calls", "epa_calls", "status_flags"):
            assert cr[k] == cm[k], (call, k, cr[k], cm[k])
        assert cm["status_flags"] == 0
        bad = H.compare_manifolds(ref.get_manifolds(), mine.get_manifolds())
        assert not bad, (call, bad)
        m = mine.get_manifolds()
        assert m["num_points"].sum() > 0
    ref.close()
    mine.close()


def test_static_scratch_rejects_out_of_range_slots(gpu_lib):
    narrow_static, L = _entry()
    sc = overlapping_pairs(4)
    g = GpuWorld(sc)
    _to_pairs(g, sc.dt)
    assert narrow_static(g.h, STATIC_EPA_SLOTS_MAX + 1) == _abi.ERR_CAPACITY
    assert b"exceeds" in L.jbgpu_last_error()
    assert narrow_static(g.h, 0) == _abi.ERR_INVALID_ARGUMENT
    assert narrow_static(g.h, 1) == 0
    g.close()
