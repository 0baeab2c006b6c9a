"""Compound shapes and triangle meshes (CompoundCollisionAlgorithm, ConvexConcaveCollisionAlgorithm
over BvhTriangleMeshShape's quantized OptimizedBvh).

CPU: the library's tree equals the oracle's node for node, the oracle's walk reports exactly the
leaves a brute-force quantized overlap test finds (in node order), compound inertia agrees three
ways, compound pairs carry one key per child combination, and the oracle's terrain and compound
scenes stay finite and above the ground.  GPU: stage by stage and closed loop bit-exact against
the oracle, the range-part solver in lockstep, and queries that reach a compound or a mesh are
reported as unsupported."""
import ctypes as C

import numpy as np
import pytest

from jbgpu import _abi, lib as jl, scenes
from jbgpu.lib import GpuWorld

import harness as H
import pyoracle

F = np.float32


def _meshes():
    rng = np.random.Generator(np.random.PCG64(5))
    out = [scenes.terrain_mesh(4, 4, 8.0, seed=1), scenes.terrain_mesh(24, 24, 24.0, seed=2),
           scenes.terrain_mesh(7, 13, 30.0, amp=4.0, seed=3)]
    # a triangle soup far from the origin, some triangles flat in an axis (MIN_AABB_DIMENSION widening)
    v = (rng.uniform(-5, 5, (300, 3)) + np.array([1000.0, -200.0, 50.0])).astype(F)
    v[:60, 1] = F(-200.0)
    idx = rng.integers(0, 300, (400, 3)).astype(np.int32)
    idx[:40] = np.stack([np.arange(0, 40), np.arange(1, 41), np.arange(2, 42)], 1)   # flat in y
    out.append({"type": _abi.SHAPE_TRIANGLE_MESH, "params": (0.0, 0.0, 0.0, 0.0), "points": v, "indices": idx})
    one = {"type": _abi.SHAPE_TRIANGLE_MESH, "params": (0.02, 0.0, 0.0, 0.0),
           "points": np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], F), "indices": np.array([[0, 2, 1]], np.int32)}
    out.append(one)
    # BvhTriangleMeshShape.setLocalScaling: a scaling that rebuilds the tree, and one within
    # SIMD_EPSILON (squared) of (1, 1, 1) that the reference ignores
    out.append(scenes.terrain_mesh(24, 24, 24.0, seed=2, scaling=(1.5, 0.6, 0.8)))
    out.append(scenes.terrain_mesh(7, 13, 30.0, amp=4.0, seed=3, scaling=(1.0001, 1.0, 0.9999)))
    return out


NMESH = 7


def _scaled_points(mesh):
    """The vertices as the reference reads them (VertexData.getTriangle: times the scaling, set by
    setLocalScaling only when it is more than SIMD_EPSILON (squared) away from (1, 1, 1))."""
    p = np.asarray(mesh["points"], F)
    s = np.asarray(mesh["params"][1:4], F)
    if not s.any():
        return p
    d = F(1) - s
    if not (F(d[0] * d[0] + d[1] * d[1]) + F(d[2] * d[2]) > F(1.1920929e-7)):
        return p
    return (p * s).astype(F)


def _quantizer(mesh):
    """OptimizedBvh.setQuantizationValues / quantizeWithClamp in binary32 (for the brute force)."""
    p = _scaled_points(mesh)[np.asarray(mesh["indices"]).reshape(-1)]
    bmin, bmax = p.min(0) - F(1), p.max(0) + F(1)
    q = F(65535.0) / (bmax - bmin)

    def quant(x):
        c = np.minimum(np.maximum(np.asarray(x, F), bmin), bmax)
        v = (c - bmin) * q
        return (np.floor(v + F(0.5)).astype(np.int64) & 0xFFFF)
    return quant


def _unpack(nodes):
    n = nodes.astype(np.int64) & 0xFFFFFFFF
    qmin = np.stack([n[:, 0] & 0xFFFF, n[:, 0] >> 16, n[:, 1] & 0xFFFF], 1)
    qmax = np.stack([n[:, 1] >> 16, n[:, 2] & 0xFFFF, n[:, 2] >> 16], 1)
    return qmin, qmax, nodes[:, 3]


@pytest.mark.parametrize("k", range(NMESH))
def test_mesh_tree_library_equals_oracle(gpu_lib, oracle_lib, k):
    mesh = _meshes()[k]
    ln, la = jl.mesh_bvh(mesh)
    on, oa = pyoracle.mesh_bvh(mesh)
    assert ln.shape == on.shape and np.array_equal(ln, on)
    assert np.array_equal(la.view(np.uint32), oa.view(np.uint32))


@pytest.mark.parametrize("k", range(NMESH))
def test_mesh_tree_structure(oracle_lib, k):
    mesh = _meshes()[k]
    nodes, aabb = pyoracle.mesh_bvh(mesh)
    nt = len(mesh["indices"])
    assert len(nodes) == 2 * nt - 1
    w = nodes[:, 3]
    assert sorted(w[w >= 0].tolist()) == list(range(nt))   # every triangle once, as a leaf

    def size(i):   # subtree size from the escape index, checked against the children's sizes
        if w[i] >= 0:
            return 1
        left = size(i + 1)
        right = size(i + 1 + left)
        assert -w[i] == 1 + left + right
        return -w[i]
    assert size(0) == len(nodes)
    p = _scaled_points(mesh)[np.asarray(mesh["indices"]).reshape(-1)]
    assert np.array_equal(aabb[:3], p.min(0)) and np.array_equal(aabb[3:], p.max(0))


def test_mesh_scaling_rebuilds_over_the_scaled_vertices(gpu_lib, oracle_lib):
    """setLocalScaling's tree is the tree of the scaled vertex array; a scaling within
    SIMD_EPSILON of (1, 1, 1) leaves the mesh as it was."""
    meshes = _meshes()
    scaled, near = meshes[5], meshes[6]
    plain = dict(scaled, params=(0.0, 0.0, 0.0, 0.0), points=_scaled_points(scaled))
    assert not np.array_equal(plain["points"], scaled["points"])
    for fn in (jl.mesh_bvh, pyoracle.mesh_bvh):
        a, b = fn(scaled), fn(plain)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
        c, d = fn(near), fn(dict(near, params=(0.0, 0.0, 0.0, 0.0)))
        assert np.array_equal(c[0], d[0]) and np.array_equal(c[1].view(np.uint32), d[1].view(np.uint32))


def test_mirror_mesh_scaling_order():
    """The mirror takes setLocalScaling before setMargin (the reference's rebuilt tree would take
    the margin into its quantization bounds otherwise) and reports the scaling the reference keeps."""
    from jbgpu import dynamics as D
    tm = scenes.terrain_mesh(4, 4, 8.0, seed=1)
    s = D.BvhTriangleMeshShape(D.TriangleIndexVertexArray(tm["indices"], tm["points"]), True)
    assert np.array_equal(s.getLocalScaling(), np.ones(3, F))
    s.setLocalScaling((1.0001, 1.0, 1.0))
    assert np.array_equal(s.getLocalScaling(), np.ones(3, F))
    s.setLocalScaling((2.0, 0.5, 1.0))
    s.setMargin(0.04)
    assert s.desc()["params"] == (0.04, 2.0, 0.5, 1.0)
    assert np.array_equal(s.getLocalScaling(), np.array([2.0, 0.5, 1.0], F))
    with pytest.raises(NotImplementedError):
        s.setLocalScaling((1.5, 1.5, 1.5))


def _deformed(mesh, seed):
    """The mesh's vertices moved (same count): heights shifted by up to 0.4 m, x and z by up to
    0.05 m, and one vertex lifted 2 m."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.asarray(mesh["points"], F).copy()
    p[:, 1] += rng.uniform(-0.4, 0.4, len(p)).astype(F)
    p[:, 0] += rng.uniform(-0.05, 0.05, len(p)).astype(F)
    p[:, 2] += rng.uniform(-0.05, 0.05, len(p)).astype(F)
    p[len(p) // 2, 1] += F(2.0)
    return p


def _static_mesh_scene(mesh):
    b = scenes._bodies(1)
    b["transform"][0] = scenes.xf12()
    return scenes.Scene("mesh_only", 1.0 / 60.0, 1, {}, [mesh], b)


@pytest.mark.parametrize("k", [1, 2, 5])
def test_oracle_refit_keeps_topology_and_requantizes(oracle_lib, k):
    """OptimizedBvh.refit in the oracle: the same nodes, every leaf the quantized box of its moved
    triangle under the new quantization (no minimum extent), every internal node the union of its
    two children, the local aabb the moved vertices' box widened by the margin."""
    mesh = dict(_meshes()[k], params=(0.03,) + tuple(_meshes()[k]["params"][1:4]))
    o = pyoracle.OracleWorld(_static_mesh_scene(mesh))
    n0, _ = o.mesh_bvh(0)
    moved = _deformed(mesh, k)
    o.refit_mesh(0, moved)
    n1, aabb = o.mesh_bvh(0)
    assert np.array_equal(n0[:, 3], n1[:, 3])
    quant = _quantizer(dict(mesh, points=moved))
    p = _scaled_points(dict(mesh, points=moved))[np.asarray(mesh["indices"]).reshape(-1, 3)]
    qmin, qmax, w = _unpack(n1)
    leaves = np.nonzero(w >= 0)[0]
    assert np.array_equal(qmin[leaves], quant(p[w[leaves]].min(1))) and np.array_equal(qmax[leaves], quant(p[w[leaves]].max(1)))
    for i in np.nonzero(w < 0)[0]:
        l = i + 1
        r = i + 2 if w[l] >= 0 else i + 1 - w[l]
        assert np.array_equal(qmin[i], np.minimum(qmin[l], qmin[r])) and np.array_equal(qmax[i], np.maximum(qmax[l], qmax[r]))
    flat = p.reshape(-1, 3)
    assert np.array_equal(aabb[:3], flat.min(0) - F(0.03)) and np.array_equal(aabb[3:], flat.max(0) + F(0.03))
    with pytest.raises(ValueError):
        o.refit_mesh(0, moved[:-1])


@pytest.mark.parametrize("k", range(NMESH))
def test_mesh_walk_reports_overlapping_leaves_in_node_order(oracle_lib, k):
    mesh = _meshes()[k]
    nodes, _ = pyoracle.mesh_bvh(mesh)
    qmin, qmax, w = _unpack(nodes)
    quant = _quantizer(mesh)
    p = _scaled_points(mesh)[np.asarray(mesh["indices"]).reshape(-1)]
    lo, hi = p.min(0), p.max(0)
    rng = np.random.Generator(np.random.PCG64(k))
    for _ in range(40):
        c = rng.uniform(lo - 1, hi + 1).astype(F)
        e = rng.uniform(0.0, 0.3, 3).astype(F) * (hi - lo + 1)
        mn, mx = c - e, c + e
        got = pyoracle.mesh_query(mesh, mn, mx)
        a, b = quant(mn), quant(mx)
        ov = np.all((a <= qmax) & (b >= qmin), axis=1)
        want = w[(w >= 0) & ov]
        assert np.array_equal(got, want)


def test_compound_inertia_three_ways(gpu_lib, oracle_lib):
    rng = np.random.Generator(np.random.PCG64(3))
    for s, m, inertia in scenes._compound_kinds(rng, 8):
        a = jl.shape_local_inertia(s, float(m))
        b = pyoracle.shape_local_inertia(s, float(m))
        assert np.array_equal(a.view(np.uint32), inertia.view(np.uint32)), (a, inertia)
        assert np.array_equal(b.view(np.uint32), inertia.view(np.uint32)), (b, inertia)


def test_compound_child_limit(gpu_lib):
    child = {"type": _abi.SHAPE_SPHERE, "params": (0.1, 0.0, 0.0, 0.0), "points": None}
    ok = {"type": _abi.SHAPE_COMPOUND, "params": (0.0, 0.0, 0.0, 0.0), "points": None,
          "children": [(child, scenes.xf12(None, (i, 0, 0))) for i in range(_abi.COMPOUND_MAX_CHILDREN)]}
    jl.shape_local_inertia(ok, 1.0)
    bad = dict(ok, children=ok["children"] + [(child, scenes.xf12(None, (20, 0, 0)))])
    d = scenes.shape_desc_array([bad])
    out = np.zeros(3, np.float32)
    assert jl.lib().jbgpu_shape_local_inertia(C.byref(d[0]), 1.0, out.ctypes.data_as(_abi.f32p)) == \
        _abi.ERR_INVALID_ARGUMENT
    nested = dict(ok, children=[(ok, scenes.xf12())])
    d = scenes.shape_desc_array([nested])
    assert jl.lib().jbgpu_shape_local_inertia(C.byref(d[0]), 1.0, out.ctypes.data_as(_abi.f32p)) == \
        _abi.ERR_UNSUPPORTED


def _subs(sc, a, b):
    n = [len(sc.shapes[sc.bodies["shape"][x]].get("children") or []) or 1 for x in (a, b)]
    return n[0] * n[1]


def test_compound_pairs_one_key_per_child_combination(oracle_lib):
    sc = scenes.compounds(12, 6, seed=4)
    o = pyoracle.OracleWorld(sc)
    for _ in range(90):
        o.step(sc.dt)
    keys = o.get_pairs()
    assert len(keys) and np.all(np.diff(keys.astype(np.uint64)) > 0)
    owner, partner, sub = keys >> np.uint64(32), keys & np.uint64(0xFFFFFF), (keys >> np.uint64(24)) & np.uint64(0xFF)
    per = {}
    for a, b, s in zip(owner.tolist(), partner.tolist(), sub.tolist()):
        per.setdefault((a, b), []).append(s)
    assert any(len(v) > 1 for v in per.values())
    for (a, b), v in per.items():
        assert sorted(v) == list(range(_subs(sc, a, b)))


@pytest.mark.parametrize("which", ["terrain", "compounds"])
def test_oracle_f3_scenes_stay_on_the_ground(oracle_lib, which):
    if which == "terrain":
        sc = scenes.terrain(40, compounds=8, seed=2)
        floor = F(sc.shapes[0]["points"][:, 1].min()) - F(0.5)
    else:
        sc = scenes.compounds(30, 10, seed=2)
        floor = F(-0.1)
    o = pyoracle.OracleWorld(sc)
    for _ in range(sc.steps):
        o.step(sc.dt)
    t = o.get_state()["transform"]
    assert np.isfinite(t).all()
    assert (t[1:, 10] > floor).all()
    c = o.counters()
    assert c["contacts"] > len(sc.bodies) // 2


# ---- GPU -------------------------------------------------------------------------------------
STAGES = [_abi.STAGE_PREDICT, _abi.STAGE_AABB, _abi.STAGE_PAIRS, _abi.STAGE_NARROWPHASE, _abi.STAGE_ISLANDS,
          _abi.STAGE_SOLVE, _abi.STAGE_INTEGRATE, _abi.STAGE_ACTIVATION]

SCENES = {
    "terrain": lambda: scenes.terrain(40, seed=1),
    "terrain_compounds": lambda: scenes.terrain(30, compounds=12, seed=2),
    "compounds": lambda: scenes.compounds(30, 10, seed=3),
    "terrain_margin": lambda: _with_mesh_margin(scenes.terrain(30, compounds=4, seed=5), 0.05),
    "terrain_scaled": lambda: _with_mesh_margin(scenes.terrain(30, compounds=4, seed=7, mesh_scaling=(1.3, 0.7, 1.1)),
                                                0.02),
}


def _with_mesh_margin(sc, m):
    sc.shapes[0] = dict(sc.shapes[0], params=(m,) + tuple(sc.shapes[0]["params"][1:4]))
    return sc


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("warm", [0, 60, 150])
def test_f3_stage_by_stage_bit_exact(gpu_lib, oracle_lib, name, warm):
    sc = SCENES[name]()
    ref = pyoracle.OracleWorld(sc)
    for _ in range(warm):
        ref.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    H.copy_world(ref, o)
    H.copy_world(ref, g)
    o.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    g.stage(_abi.STAGE_APPLY_GRAVITY, sc.dt)
    for st in STAGES:
        H.copy_world(o, g)
        o.stage(st, sc.dt)
        g.stage(st, sc.dt)
        bs = H.compare_state(o.get_state(), g.get_state())
        bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
        assert not bs and not bm, (st, bs, bm)
        if st == _abi.STAGE_NARROWPHASE:
            co, cg = o.counters(), g.counters()
            assert (co["gjk_calls"], co["epa_calls"]) == (cg["gjk_calls"], cg["epa_calls"])
        if st == _abi.STAGE_SOLVE:
            assert np.array_equal(o.solver_order(), g.solver_order())
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(SCENES))
def test_f3_closed_loop_bit_exact(gpu_lib, oracle_lib, name):
    sc = SCENES[name]()
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    for s in range(sc.steps):
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    co, cg = o.counters(), g.counters()
    for k in ("pairs", "manifolds", "contacts", "solver_manifolds", "solver_rows", "gjk_calls", "epa_calls"):
        assert co[k] == cg[k], (k, co[k], cg[k])
    assert cg["status_flags"] == 0
    assert co["contacts"] > 0
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["terrain_compounds", "compounds"])
def test_f3_range_parts_lockstep_bit_exact(gpu_lib, oracle_lib, name):
    sc = SCENES[name]()
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc, config=_abi.default_config(**dict(sc.config, solver_parts=3)))
    for s in range(120):
        g.step(sc.dt)
        o.set_explicit_order(g.solver_order())
        o.step(sc.dt)
        assert o.counters()["status_flags"] == 0, s
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    g.close()


@pytest.mark.gpu
def test_f3_batched_worlds_equal_solo(gpu_lib):
    """Three terrain/compound worlds batched: each world's bodies end where the same world
    stepped alone leaves them."""
    parts = [scenes.terrain(12, compounds=4, seed=s) for s in (7, 8, 9)]
    shapes, bodies, wid = [], [], []
    for w, sc in enumerate(parts):
        b = sc.bodies.copy()
        b["shape"] += len(shapes)
        b["world"] = w
        shapes += sc.shapes
        bodies.append(b)
        wid.append(np.full(len(b), w, np.int32))
    batch = scenes.Scene("f3_batch", parts[0].dt, 90, parts[0].config, shapes, np.concatenate(bodies),
                         world_of_body=np.concatenate(wid))
    g = GpuWorld(batch)
    for _ in range(90):
        g.step(batch.dt)
    tb = g.get_state()["transform"]
    g.close()
    off = 0
    for sc in parts:
        s = GpuWorld(sc)
        for _ in range(90):
            s.step(sc.dt)
        ts = s.get_state()["transform"]
        s.close()
        assert np.array_equal(tb[off:off + len(ts)].view(np.uint32), ts.view(np.uint32))
        off += len(ts)


@pytest.mark.gpu
def test_f3_dynamic_mesh_rejected(gpu_lib):
    bad = scenes.terrain(2, seed=1)           # a dynamic triangle-mesh body
    bad.bodies["mass"][0] = 1.0
    with pytest.raises(jl.JbgpuError) as e:
        GpuWorld(bad)
    assert e.value.code == _abi.ERR_INVALID_ARGUMENT


def _same(a, b):
    return np.array_equal(a.view(np.uint8).reshape(len(a), -1), b.view(np.uint8).reshape(len(b), -1))


def _ray_tri(o, d, tri):
    """Moller-Trumbore in float64: the ray parameter of a hit, or inf."""
    e1, e2 = tri[1] - tri[0], tri[2] - tri[0]
    p = np.cross(d, e2)
    det = e1 @ p
    if abs(det) < 1e-12:
        return np.inf
    t0 = o - tri[0]
    u = (t0 @ p) / det
    q = np.cross(t0, e1)
    v = (d @ q) / det
    t = (e2 @ q) / det
    return t if (u >= 0 and v >= 0 and u + v <= 1 and 0 <= t <= 1) else np.inf


def test_oracle_rays_hit_the_mesh_and_compound_children(oracle_lib):
    sc = scenes.terrain(4, compounds=2, seed=3)
    o = pyoracle.OracleWorld(sc)
    tm = sc.shapes[0]
    tris = np.asarray(tm["points"], np.float64)[np.asarray(tm["indices"])]
    rng = np.random.Generator(np.random.PCG64(2))
    frm = np.stack([rng.uniform(-7, 7, 64), np.full(64, 30.0), rng.uniform(-7, 7, 64)], 1).astype(F)
    to = frm.copy()
    to[:, 1] = -30.0
    to[:, 0] += rng.uniform(-2, 2, 64).astype(F)
    h = o.ray_test(frm, to)
    ground = np.nonzero(h["body"] == 0)[0]
    assert len(ground) > 40
    for k in ground:
        d = to[k].astype(np.float64) - frm[k]
        want = min(_ray_tri(frm[k].astype(np.float64), d, t) for t in tris)
        assert abs(h["fraction"][k] - want) < 1e-5
        assert h["normal"][k][1] > 0
    # a compound: rays at its body origin hit a child at most 0.01 before the child's surface
    comp = [i for i in range(1, len(sc.bodies)) if sc.shapes[sc.bodies["shape"][i]]["type"] == _abi.SHAPE_COMPOUND]
    for i in comp:
        c = sc.bodies["transform"][i, 9:12]
        r = o.ray_test((c + np.array([0, 10, 0], F))[None], (c - np.array([0, 10, 0], F))[None])
        assert r["body"][0] == i


def _height(tm, x, z):
    """The terrain surface's height under (x, z) (float64 barycentric over the cell's triangles)."""
    tris = np.asarray(tm["points"], np.float64)[np.asarray(tm["indices"])]
    for t in tris:
        a, b, c = t[0][[0, 2]], t[1][[0, 2]], t[2][[0, 2]]
        m = np.array([b - a, c - a]).T
        if abs(np.linalg.det(m)) < 1e-12:
            continue
        u, v = np.linalg.solve(m, np.array([x, z]) - a)
        if u >= -1e-9 and v >= -1e-9 and u + v <= 1 + 1e-9:
            return t[0][1] + u * (t[1][1] - t[0][1]) + v * (t[2][1] - t[0][1])
    return None


def test_oracle_sweeps_hit_the_mesh(oracle_lib):
    """A sphere of radius 0.3 swept straight down onto the terrain stops with its centre about 0.3
    from the reported point, which lies on the mesh."""
    sc = scenes.terrain(2, seed=3)
    o = pyoracle.OracleWorld(sc)
    tm = sc.shapes[0]
    cast = next(i for i, x in enumerate(sc.shapes) if x["type"] == _abi.SHAPE_SPHERE)
    r = sc.shapes[cast]["params"][0]
    rng = np.random.Generator(np.random.PCG64(5))
    m = 32
    xz = rng.uniform(-6, 6, (m, 2)).astype(F)
    fr = np.stack([scenes.xf12(None, (x, 30.0, z)) for x, z in xz])
    to = np.stack([scenes.xf12(None, (x, -30.0, z)) for x, z in xz])
    h, planes = o.convex_sweep(cast, fr, to)
    assert planes == 0
    ground = np.nonzero(h["body"] == 0)[0]    # the other sweeps meet one of the scene's two bodies
    assert len(ground) >= m - 4
    for k in ground:
        c = fr[k, 9:12] + h["fraction"][k] * (to[k, 9:12] - fr[k, 9:12])
        p = h["point"][k].astype(np.float64)
        assert abs(np.linalg.norm(c - p) - r) < 0.02
        y = _height(tm, p[0], p[2])
        assert y is not None and abs(y - p[1]) < 1e-3
        assert h["normal"][k][1] > 0.5


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [0, 90])
def test_f3_sweeps_bit_exact_on_the_mesh(gpu_lib, oracle_lib, steps):
    sc = scenes.terrain(40, compounds=16, seed=6)
    g = GpuWorld(sc)
    for _ in range(steps):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=False)
    rng = np.random.Generator(np.random.PCG64(12))
    casts = [i for i, x in enumerate(sc.shapes) if x["type"] in (_abi.SHAPE_BOX, _abi.SHAPE_SPHERE, _abi.SHAPE_CAPSULE,
                                                                   _abi.SHAPE_CONVEX_HULL)][:4]
    kinds = np.array([sc.shapes[x]["type"] for x in sc.bodies["shape"]])
    on_mesh = 0
    for shape in casts:
        m = 256
        a = rng.uniform(-7, 7, (m, 3)).astype(F)
        a[:, 1] = rng.uniform(2, 10, m)
        b = a + rng.uniform(-3, 3, (m, 3)).astype(F)
        b[:, 1] = rng.uniform(-3, 4, m)
        Ra, Rb = scenes.random_rotations(rng, m), scenes.random_rotations(rng, m)
        fr = np.concatenate([Ra.reshape(m, 9), a], 1).astype(F)
        to = np.concatenate([Rb.reshape(m, 9), b], 1).astype(F)
        hg = g.convex_sweep_test(shape, fr, to)
        ho, planes = o.convex_sweep(shape, fr, to)
        assert planes == 0 and _same(ho, hg), (shape, np.nonzero(ho != hg)[0][:10])
        on_mesh += (kinds[hg["body"][hg["body"] >= 0]] == _abi.SHAPE_TRIANGLE_MESH).sum()
    assert on_mesh > 200
    g.close()


@pytest.mark.gpu
def test_f3_ccd_on_the_mesh_closed_loop_bit_exact(gpu_lib, oracle_lib):
    """CCD motion clamping of fast convex bodies onto the triangle-mesh terrain (the sweep's mesh
    branch) and onto compound bodies."""
    sc = scenes.terrain(30, compounds=6, seed=10)
    sc.bodies["linear_velocity"][1::2] = (0.0, -40.0, 0.0)
    sc.meta["ccd"] = {"bodies": list(range(1, len(sc.bodies))), "threshold": 0.05, "radius": 0.1}
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    clamped = 0
    for s in range(90):
        o.step(sc.dt)
        g.step(sc.dt)
        clamped += g.counters()["ccd_clamped"]
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            assert not bs, (s, bs)
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    assert clamped > 0 and g.counters()["status_flags"] == 0
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [0, 90])
def test_f3_rays_bit_exact(gpu_lib, oracle_lib, steps):
    sc = scenes.terrain(40, compounds=16, seed=6)
    g = GpuWorld(sc)
    for _ in range(steps):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=False)
    rng = np.random.Generator(np.random.PCG64(8))
    n = 4096
    frm = rng.uniform(-8, 8, (n, 3)).astype(F)
    frm[:, 1] = rng.uniform(-1, 12, n)
    to = rng.uniform(-8, 8, (n, 3)).astype(F)
    to[:, 1] = rng.uniform(-3, 12, n)
    to[: n // 2, :] = frm[: n // 2]
    to[: n // 2, 1] = -3.0                     # half straight down
    hg = g.ray_test(frm, to)
    ho = o.ray_test(frm, to)
    assert _same(ho, hg), np.nonzero(ho != hg)[0][:10]
    kinds = np.array([sc.shapes[x]["type"] for x in sc.bodies["shape"]])
    hit = hg["body"][hg["body"] >= 0]
    assert (kinds[hit] == _abi.SHAPE_TRIANGLE_MESH).sum() > 500
    assert (kinds[hit] == _abi.SHAPE_COMPOUND).sum() > 20
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [0, 60])
def test_f3_sweeps_bit_exact_on_compounds(gpu_lib, oracle_lib, steps):
    sc = scenes.compounds(30, 12, seed=7)
    g = GpuWorld(sc)
    for _ in range(steps):
        g.step(sc.dt)
    o = pyoracle.OracleWorld(sc)
    H.copy_world(g, o, manifolds=False)
    rng = np.random.Generator(np.random.PCG64(4))
    casts = [i for i, x in enumerate(sc.shapes) if x["type"] in (_abi.SHAPE_BOX, _abi.SHAPE_SPHERE, _abi.SHAPE_CAPSULE,
                                                                   _abi.SHAPE_CONVEX_HULL)][:4]
    kinds = np.array([sc.shapes[x]["type"] for x in sc.bodies["shape"]])
    on_compounds = 0
    for shape in casts:
        m = 256
        a = rng.uniform(-4, 4, (m, 3)).astype(F)
        a[:, 1] = rng.uniform(0.2, 8, m)
        b = rng.uniform(-4, 4, (m, 3)).astype(F)
        b[:, 1] = rng.uniform(0.2, 8, m)
        R = scenes.random_rotations(rng, m)
        fr = np.concatenate([R.reshape(m, 9), a], 1).astype(F)
        to = np.concatenate([R.reshape(m, 9), b], 1).astype(F)
        hg = g.convex_sweep_test(shape, fr, to, mask=~2)
        ho, planes = o.convex_sweep(shape, fr, to, mask=~2)
        assert planes == 0 and _same(ho, hg), (shape, np.nonzero(ho != hg)[0][:10])
        on_compounds += (kinds[hg["body"][hg["body"] >= 0]] == _abi.SHAPE_COMPOUND).sum()
    assert on_compounds > 50
    g.close()


@pytest.mark.gpu
def test_f3_ccd_with_compounds_closed_loop_bit_exact(gpu_lib, oracle_lib):
    """CCD motion clamping where the swept bodies meet compound bodies (the sweep's compound branch);
    fast compound bodies move unclamped, as integrateTransforms sweeps convex bodies only
    (DiscreteDynamicsWorld.java:700-729)."""
    sc = scenes.compounds(20, 10, seed=9, region=(3.0, 4.0, 3.0), y0=0.5)
    # a static box for ground (a CCD sweep reaching a static plane is where the reference throws)
    sc.shapes[0] = {"type": _abi.SHAPE_BOX, "params": (20.0, 0.5, 20.0, 0.0), "points": None}
    sc.bodies["transform"][0, 9:12] = (0.0, -0.5, 0.0)
    sc.bodies["linear_velocity"][1::3] = (0.0, -25.0, 0.0)
    sc.meta["ccd"] = {"bodies": list(range(1, len(sc.bodies))), "threshold": 0.05, "radius": 0.1}
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    clamped = 0
    for s in range(90):
        o.step(sc.dt)
        g.step(sc.dt)
        clamped += g.counters()["ccd_clamped"]
        if s % 10 == 9 or s < 5:
            bs = H.compare_state(o.get_state(), g.get_state())
            assert not bs, (s, bs)
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    assert clamped > 0
    g.close()


@pytest.mark.gpu
def test_mirror_compound_on_mesh_reads_like_the_reference(gpu_lib, oracle_lib):
    """The reference's usage through the Python mirror: a BvhTriangleMeshShape ground over a
    TriangleIndexVertexArray (setLocalScaling, then setMargin), CompoundShape dumbbells built with
    addChildShape and a box; two seconds of stepSimulation with the ground deformed in place and
    refitTree called after the first.  The same world given to the oracle ends bit-identical."""
    from jbgpu import dynamics as D
    tm = scenes.terrain_mesh(8, 8, 12.0, seed=4)
    world = D.DiscreteDynamicsWorld()
    world.setGravity((0.0, -9.81, 0.0))
    ground_shape = D.BvhTriangleMeshShape(D.TriangleIndexVertexArray(tm["indices"], tm["points"]), True)
    ground_shape.setLocalScaling((1.2, 0.8, 1.1))
    ground_shape.setMargin(0.01)
    ground = D.RigidBody(D.RigidBodyConstructionInfo(0.0, None, ground_shape))
    world.addRigidBody(ground)
    bell = D.CompoundShape()
    bell.addChildShape(D.Transform(origin=(-0.6, 0.0, 0.0)), D.SphereShape(0.3))
    bell.addChildShape(D.Transform(origin=(0.6, 0.0, 0.0)), D.SphereShape(0.3))
    bell.addChildShape(D.Transform(basis=scenes.rot_z(np.pi / 2)), D.CapsuleShape(0.1, 1.2))
    box = D.BoxShape((0.4, 0.3, 0.2))
    specs = [(bell, 2.0, (0.0, 4.0, 0.0)), (bell, 2.0, (0.5, 6.0, 0.3)), (box, 1.0, (-0.8, 5.0, -0.4))]
    for shape, m, pos in specs:
        info = D.RigidBodyConstructionInfo(m, None, shape, shape.calculateLocalInertia(m))
        info.startWorldTransform = D.Transform(basis=scenes.rot_x(0.4), origin=pos)
        world.addRigidBody(D.RigidBody(info))
    for _ in range(60):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    # the terrain deformed in place, then refitTree (the mesh interface's vertices are the array)
    verts = ground_shape.getMeshInterface().vertices
    orig = verts.copy()
    moved = orig.copy()
    moved[:, 1] = moved[:, 1] * F(0.9) + F(0.05)   # the ground flattened a little and raised 5 cm
    verts[:] = moved
    ground_shape.refitTree(None, None)
    for _ in range(60):
        world.stepSimulation(1.0 / 60.0, 1, 1.0 / 60.0)
    g = world._g
    # the same world on the oracle
    b = scenes._bodies(4)
    b["shape"] = [0, 1, 1, 2]
    b["mass"] = [0.0, 2.0, 2.0, 1.0]
    b["local_inertia"][1:3] = bell.calculateLocalInertia(2.0)
    b["local_inertia"][3] = box.calculateLocalInertia(1.0)
    for k, (_, _, pos) in enumerate(specs):
        b["transform"][k + 1] = scenes.xf12(scenes.rot_x(0.4), pos)
    sc = scenes.Scene("mirror_f3", 1.0 / 60.0, 120, {"gravity": (0.0, -9.81, 0.0)},
                      [ground_shape.desc(), bell.desc(), box.desc()], b)
    sc.shapes[0] = dict(sc.shapes[0], points=orig)   # the vertices it was built over
    o = pyoracle.OracleWorld(sc, config=_abi.default_config(gravity=(0.0, -9.81, 0.0)))
    for _ in range(60):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    o.refit_mesh(0, moved)
    for _ in range(60):
        o.step_simulation(1.0 / 60.0, 1, 1.0 / 60.0)
    assert not H.compare_state(o.get_state(), g.get_state())
    assert not H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
    assert o.counters()["contacts"] > 0
    world.close()


@pytest.mark.gpu
@pytest.mark.parametrize("scaled", [False, True])
def test_refit_tree_and_closed_loop_bit_exact(gpu_lib, oracle_lib, scaled):
    """BvhTriangleMeshShape.refitTree on a terrain under falling and resting bodies, twice: the
    library's refitted tree equals the oracle's node for node, and the worlds stay bit-identical
    through the refits (updateSingleAabb of the static mesh body included)."""
    sc = _with_mesh_margin(scenes.terrain(30, compounds=4, seed=11, mesh_scaling=(1.2, 0.8, 1.1) if scaled else
                                          (0.0, 0.0, 0.0)), 0.02)
    o = pyoracle.OracleWorld(sc)
    g = GpuWorld(sc)
    mesh = sc.shapes[0]
    for s in range(sc.steps):
        if s in (40, 120):
            moved = _deformed(dict(mesh, points=mesh["points"] if s == 40 else moved), s)
            o.refit_mesh(0, moved)
            g.refit_mesh(0, moved)
            on, oa = o.mesh_bvh(0)
            gn, ga = g.mesh_bvh(0)
            assert np.array_equal(on, gn) and np.array_equal(oa.view(np.uint32), ga.view(np.uint32))
        o.step(sc.dt)
        g.step(sc.dt)
        if s % 10 == 9:
            bs = H.compare_state(o.get_state(), g.get_state())
            bm = H.compare_manifolds(o.get_manifolds(), g.get_manifolds())
            assert not bs and not bm, (s, bs, bm)
    assert g.counters()["status_flags"] == 0 and o.counters()["contacts"] > 0
    with pytest.raises(jl.JbgpuError):
        g.refit_mesh(0, moved[:-1])
    with pytest.raises(jl.JbgpuError):
        g.refit_mesh(1, moved)
    g.close()
