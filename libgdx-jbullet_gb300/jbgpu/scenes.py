"""Seeded synthetic scenes for the rigid-body step.

The reference ships no benchmark scene or dataset; these generators build the five
workloads the step is measured on (boxes on a plane; 100k mixed spheres/boxes/capsules;
20k convex hulls; 4,096 batched worlds; pyramids for the warm-start study) from a PCG64
stream, so the same seed yields the same bodies on every machine.

Mass properties follow the reference's CollisionShape.calculateLocalInertia, evaluated in
binary32 with the reference's operation order (collision/shapes/BoxShape.java:153-167,
SphereShape.java:72-76, CapsuleShape.java:125-153, PolyhedralConvexShape.java:133-159),
so that the oracle and the GPU library receive identical inputs.
"""
from dataclasses import dataclass, field

import numpy as np

from . import _abi

F = np.float32

BODY_DTYPE = np.dtype([
    ("mass", "<f4"), ("shape", "<i4"), ("transform", "<f4", (12,)), ("local_inertia", "<f4", (3,)),
    ("linear_damping", "<f4"), ("angular_damping", "<f4"), ("friction", "<f4"), ("restitution", "<f4"),
    ("linear_sleeping_threshold", "<f4"), ("angular_sleeping_threshold", "<f4"),
    ("linear_velocity", "<f4", (3,)), ("angular_velocity", "<f4", (3,)),
    ("collision_group", "<i4"), ("collision_mask", "<i4"), ("world", "<i4"),
    ("collision_flags", "<i4"), ("activation_state", "<i4"),
])
assert BODY_DTYPE.itemsize == 136


@dataclass
class Scene:
    name: str
    dt: float
    steps: int
    config: dict
    shapes: list                      # dicts: type, params (4 floats), points (n,3) float32 or None;
                                      # meshes add indices (m,3) int32, compounds children: a list of
                                      # (shape dict, transform 12 floats)
    bodies: np.ndarray                # BODY_DTYPE records, insertion order (uid = index + 1)
    world_of_body: np.ndarray = None  # batched scenes: world index per body
    meta: dict = field(default_factory=dict)

    @property
    def n_bodies(self):
        return len(self.bodies)

    def shape_descs(self):
        """ctypes array of ShapeDesc (keeps point buffers alive on the returned object)."""
        return shape_desc_array(self.shapes)

    def body_descs_ptr(self):
        b = np.ascontiguousarray(self.bodies)
        return b, b.ctypes.data_as(_abi.C.POINTER(_abi.BodyDesc))


def _fill_desc(d, s, keep):
    d.type = s["type"]
    d.params[:] = tuple(float(x) for x in s["params"])
    d.points, d.num_points, d.indices, d.num_triangles = None, 0, None, 0
    d.children, d.child_transforms, d.num_children = None, None, 0
    if s.get("points") is not None:
        p = np.ascontiguousarray(s["points"], dtype=np.float32).reshape(-1, 3)
        keep.append(p)
        d.points = p.ctypes.data_as(_abi.f32p)
        d.num_points = len(p)
    if s.get("indices") is not None:
        ix = np.ascontiguousarray(s["indices"], dtype=np.int32).reshape(-1, 3)
        keep.append(ix)
        d.indices = ix.ctypes.data_as(_abi.C.POINTER(_abi.C.c_int32))
        d.num_triangles = len(ix)
    if s.get("children"):
        ch = (_abi.ShapeDesc * len(s["children"]))()
        xf = np.ascontiguousarray([np.asarray(t, np.float32).reshape(12) for _, t in s["children"]], np.float32)
        for k, (c, _) in enumerate(s["children"]):
            _fill_desc(ch[k], c, keep)
        keep.extend([ch, xf])
        d.children = _abi.C.cast(ch, _abi.C.POINTER(_abi.ShapeDesc))
        d.child_transforms = xf.ctypes.data_as(_abi.f32p)
        d.num_children = len(s["children"])


def shape_desc_array(shapes):
    """ctypes array of ShapeDesc for a list of shape dicts (the buffers it points into are kept
    alive on the array)."""
    arr = (_abi.ShapeDesc * len(shapes))()
    keep = []
    for i, s in enumerate(shapes):
        _fill_desc(arr[i], s, keep)
    arr._keep = keep
    return arr


# ---- binary32 mass properties (reference operation order) --------------------------------
def box_inertia(mass, half_extents, margin=F(0.04)):
    he = np.asarray(half_extents, F)
    dims = he * F(1) - margin                      # BoxShape ctor: implicit dims
    hm = dims + margin                             # getHalfExtentsWithMargin
    lx, ly, lz = F(2) * hm[0], F(2) * hm[1], F(2) * hm[2]
    m12 = F(mass) / F(12)
    return np.array([m12 * (ly * ly + lz * lz), m12 * (lx * lx + lz * lz), m12 * (lx * lx + ly * ly)], F)


def sphere_inertia(mass, r):
    e = F(0.4) * F(mass) * F(r) * F(r)
    return np.array([e, e, e], F)


def capsule_inertia(mass, r, height):
    r = F(r)
    hh = F(0.5) * F(height)
    he = np.array([r, r + hh, r], F)
    margin = F(0.04)
    lx, ly, lz = F(2) * (he[0] + margin), F(2) * (he[1] + margin), F(2) * (he[2] + margin)
    x2, y2, z2 = lx * lx, ly * ly, lz * lz
    sm = F(mass) * F(0.08333333)
    return np.array([sm * (y2 + z2), sm * (x2 + z2), sm * (x2 + y2)], F)


def hull_local_aabb(points, margin=F(0.04)):
    """PolyhedralConvexShape.recalcLocalAabb (strict > argmax in point order)."""
    p = np.asarray(points, F)
    mx = np.empty(3, F)
    mn = np.empty(3, F)
    for i in range(3):
        # dot with a unit axis: x*1 + y*0 + z*0 has the value of the coordinate
        mx[i] = p[int(np.argmax(p[:, i])), i] + margin
        mn[i] = p[int(np.argmax(-p[:, i])), i] - margin
    return mn, mx


def hull_inertia(mass, points, margin=F(0.04)):
    mn, mx = hull_local_aabb(points, margin)
    lhe = (mx - mn) * F(0.5) + margin              # transformAabb with the identity transform
    lc = (mx + mn) * F(0.5)
    amin, amax = lc - lhe, lc + lhe
    he = (amax - amin) * F(0.5)
    lx, ly, lz = F(2) * (he[0] + margin), F(2) * (he[1] + margin), F(2) * (he[2] + margin)
    x2, y2, z2 = lx * lx, ly * ly, lz * lz
    sm = F(mass) * F(0.08333333)
    return np.array([y2 + z2, x2 + z2, x2 + y2], F) * sm


# ---- helpers ------------------------------------------------------------------------------
def random_rotations(rng, n):
    """Uniform rotations from normalised 4-D Gaussians, as row-major 3x3 bases (float32)."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z); R[:, 0, 1] = 2 * (x * y - w * z); R[:, 0, 2] = 2 * (x * z + w * y)
    R[:, 1, 0] = 2 * (x * y + w * z); R[:, 1, 1] = 1 - 2 * (x * x + z * z); R[:, 1, 2] = 2 * (y * z - w * x)
    R[:, 2, 0] = 2 * (x * z - w * y); R[:, 2, 1] = 2 * (y * z + w * x); R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R.astype(F)


def _bodies(n):
    b = np.zeros(n, BODY_DTYPE)
    b["friction"] = 0.5
    b["linear_sleeping_threshold"] = 0.8
    b["angular_sleeping_threshold"] = 1.0
    b["collision_group"] = -1
    b["collision_mask"] = -1
    b["transform"][:, 0] = 1
    b["transform"][:, 4] = 1
    b["transform"][:, 8] = 1
    return b


def _plane_body(shape_id):
    b = _bodies(1)
    b["shape"] = shape_id
    return b


PLANE = {"type": _abi.SHAPE_STATIC_PLANE, "params": (0.0, 1.0, 0.0, 0.0), "points": None}


def _set_transforms(b, R, pos):
    b["transform"][:, :9] = R.reshape(-1, 9)
    b["transform"][:, 9:] = pos.astype(F)


# ---- the five workloads -------------------------------------------------------------------
def boxes_on_plane(n=1000, seed=0, region=(20.0, 50.0, 20.0), y0=1.0, steps=300):
    """1,000 unit boxes (half-extent 0.5, mass 1, friction 0.5, restitution 0), uniform in a
    20x50x20 m region above a static plane y=0, uniform random orientations, at rest;
    gravity -9.81, 10 PGS iterations, warm start 0.85, dt 1/60."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE), {"type": _abi.SHAPE_BOX, "params": (0.5, 0.5, 0.5, 0.0), "points": None}]
    b = _bodies(n)
    b["shape"] = 1
    b["mass"] = 1.0
    b["local_inertia"] = box_inertia(1.0, (0.5, 0.5, 0.5))
    pos = np.stack([rng.uniform(-region[0] / 2, region[0] / 2, n), rng.uniform(y0, y0 + region[1], n),
                    rng.uniform(-region[2] / 2, region[2] / 2, n)], 1)
    _set_transforms(b, random_rotations(rng, n), pos)
    bodies = np.concatenate([_plane_body(0), b])
    return Scene("boxes_on_plane_%d" % n, 1.0 / 60.0, steps, {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10},
                 shapes, bodies, meta={"seed": seed})


def mixed_100k(n=100_000, seed=0, region=(200.0, 100.0, 200.0), y0=1.0, steps=600):
    """100,000 bodies: 40% spheres r~U[0.2,0.6], 40% boxes half-extents~U[0.2,0.6]^3,
    20% capsules r=0.25 half-height~U[0.2,0.8] (CapsuleShape(r, 2*hh)); density 1000;
    200x100x200 m region, random orientations, v~N(0,1) per axis; 10 iterations, dt 1/120."""
    rng = np.random.Generator(np.random.PCG64(seed))
    kind = rng.permutation(np.repeat(np.arange(3), [int(0.4 * n), int(0.4 * n), n - 2 * int(0.4 * n)]))
    shapes = [dict(PLANE)]
    b = _bodies(n)
    rs = rng.uniform(0.2, 0.6, n)
    he = rng.uniform(0.2, 0.6, (n, 3))
    hh = rng.uniform(0.2, 0.8, n)
    rho = 1000.0
    for i in range(n):
        k = kind[i]
        if k == 0:
            r = F(rs[i])
            shapes.append({"type": _abi.SHAPE_SPHERE, "params": (float(r), 0.0, 0.0, 0.0), "points": None})
            m = F(rho * 4.0 / 3.0 * np.pi * float(r) ** 3)
            b["local_inertia"][i] = sphere_inertia(m, r)
        elif k == 1:
            h = he[i].astype(F)
            shapes.append({"type": _abi.SHAPE_BOX, "params": (float(h[0]), float(h[1]), float(h[2]), 0.0), "points": None})
            m = F(rho * 8.0 * float(h[0]) * float(h[1]) * float(h[2]))
            b["local_inertia"][i] = box_inertia(m, h)
        else:
            r, height = F(0.25), F(2.0 * hh[i])
            shapes.append({"type": _abi.SHAPE_CAPSULE, "params": (float(r), float(height), 0.0, 0.0), "points": None})
            m = F(rho * (np.pi * 0.25 ** 2 * float(height) + 4.0 / 3.0 * np.pi * 0.25 ** 3))
            b["local_inertia"][i] = capsule_inertia(m, r, height)
        b["mass"][i] = m
        b["shape"][i] = i + 1
    pos = np.stack([rng.uniform(-region[0] / 2, region[0] / 2, n), rng.uniform(y0, y0 + region[1], n),
                    rng.uniform(-region[2] / 2, region[2] / 2, n)], 1)
    _set_transforms(b, random_rotations(rng, n), pos)
    b["linear_velocity"] = rng.standard_normal((n, 3)).astype(F)
    bodies = np.concatenate([_plane_body(0), b])
    return Scene("mixed_%d" % n, 1.0 / 120.0, steps, {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10},
                 shapes, bodies, meta={"seed": seed, "kinds": np.concatenate([[-1], kind])})


def hulls(n=20_000, seed=0, box=60.0, y0=1.0, npts=32, steps=400):
    """n convex hulls, each the hull of 32 points uniform on an ellipsoid with semi-axes
    U[0.3,1.0]; placed by random sequential addition of non-overlapping bounding spheres in a
    60^3 m box with random orientations; density 1000 (box-inertia of the hull, as the
    reference computes it); 15 iterations, dt 1/60."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE)]
    b = _bodies(n)
    axes = rng.uniform(0.3, 1.0, (n, 3))
    radius = axes.max(axis=1)
    cell = 2.0
    grid = {}
    pos = np.zeros((n, 3))
    lo = np.array([-box / 2, y0, -box / 2])
    for i in range(n):
        for _ in range(10000):
            p = lo + rng.uniform(0, 1, 3) * box
            c = tuple((p // cell).astype(int))
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in grid.get((c[0] + dx, c[1] + dy, c[2] + dz), ()):
                            if np.sum((pos[j] - p) ** 2) < (radius[i] + radius[j]) ** 2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                break
        pos[i] = p
        grid.setdefault(c, []).append(i)
    for i in range(n):
        d = rng.standard_normal((npts, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        pts = (d * axes[i]).astype(F)
        shapes.append({"type": _abi.SHAPE_CONVEX_HULL, "params": (0.0, 0.0, 0.0, 0.0), "points": pts})
        m = F(1000.0 * 4.0 / 3.0 * np.pi * axes[i].prod())
        b["mass"][i] = m
        b["local_inertia"][i] = hull_inertia(m, pts)
        b["shape"][i] = i + 1
    _set_transforms(b, random_rotations(rng, n), pos)
    bodies = np.concatenate([_plane_body(0), b])
    return Scene("hulls_%d" % n, 1.0 / 60.0, steps, {"gravity": (0.0, -9.81, 0.0), "num_iterations": 15},
                 shapes, bodies, meta={"seed": seed})


def batched_world_counts(n_worlds=4096, seed=0, nmin=16, nmax=2048):
    """Body counts (plane excluded) of the worlds batched_worlds builds for the same arguments."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.exp(rng.uniform(np.log(nmin), np.log(nmax), n_worlds)).astype(int)


def batched_worlds(n_worlds=4096, seed=0, nmin=16, nmax=2048, sphere_frac=0.1, steps=300):
    """n_worlds independent worlds with log-uniform[16, 2048] bodies each: 90% unit boxes
    (half-extent 0.5, mass 1) and 10% spheres of radius 0.5, each world with its own plane
    and layout in a 20x50x20 m region; 10 iterations, dt 1/60.  Worlds are laid out one
    after the other (plane first in each), bodies only collide within their world."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(np.log(nmin), np.log(nmax), n_worlds)).astype(int)
    shapes = [dict(PLANE), {"type": _abi.SHAPE_BOX, "params": (0.5, 0.5, 0.5, 0.0), "points": None},
              {"type": _abi.SHAPE_SPHERE, "params": (0.5, 0.0, 0.0, 0.0), "points": None}]
    parts, wid = [], []
    for w in range(n_worlds):
        nw = int(counts[w])
        b = _bodies(nw)
        sph = rng.uniform(0, 1, nw) < sphere_frac
        b["shape"] = np.where(sph, 2, 1)
        b["mass"] = 1.0
        b["local_inertia"] = np.where(sph[:, None], sphere_inertia(1.0, 0.5), box_inertia(1.0, (0.5, 0.5, 0.5)))
        pos = np.stack([rng.uniform(-10, 10, nw), rng.uniform(1.0, 51.0, nw), rng.uniform(-10, 10, nw)], 1)
        _set_transforms(b, random_rotations(rng, nw), pos)
        parts += [_plane_body(0), b]
        wid.append(np.full(nw + 1, w, np.int32))
    bodies = np.concatenate(parts)
    bodies["world"] = np.concatenate(wid)
    return Scene("batched_%d_worlds" % n_worlds, 1.0 / 60.0, steps, {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10},
                 shapes, bodies, world_of_body=np.concatenate(wid), meta={"seed": seed, "counts": counts})


def box_stack(levels=4, seed=0, steps=120):
    """A small pyramid of unit boxes resting on the plane (a solver-hard, deterministic case)."""
    shapes = [dict(PLANE), {"type": _abi.SHAPE_BOX, "params": (0.5, 0.5, 0.5, 0.0), "points": None}]
    recs = []
    for lv in range(levels):
        for k in range(levels - lv):
            x = (k - (levels - lv - 1) / 2.0) * 1.0
            recs.append((x, 0.5 + lv * 1.0, 0.0))
    b = _bodies(len(recs))
    b["shape"] = 1
    b["mass"] = 1.0
    b["local_inertia"] = box_inertia(1.0, (0.5, 0.5, 0.5))
    b["transform"][:, 9:] = np.array(recs, F)
    bodies = np.concatenate([_plane_body(0), b])
    return Scene("box_stack_%d" % levels, 1.0 / 60.0, steps, {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10},
                 shapes, bodies, meta={"seed": seed})


def jointed_chains(chains=6, links=8, loose=24, seed=0, spacing=2.5, top=10.0, steps=240, worlds=1):
    """Chains of boxes (half-extents 0.15 x 0.45 x 0.15, 1 m long) joined end to end by point-to-
    point joints, the top link pinned to a fixed point, each chain started with a sideways
    velocity so that the chains swing into each other and into loose boxes that fall on them
    and on the plane.  meta["joints"]: {a, b, pivot_a, pivot_b} per joint (b = -1: fixed body).
    With worlds > 1 the scene is repeated in that many batch worlds (own plane each)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE), {"type": _abi.SHAPE_BOX, "params": (0.15, 0.45, 0.15, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.3, 0.3, 0.3, 0.0), "points": None}]
    side = int(np.ceil(np.sqrt(chains)))
    all_bodies, joints, wid = [], [], []
    base = 0
    for wi in range(worlds):
        plane = _plane_body(0)
        lb = _bodies(chains * links)
        lb["shape"] = 1
        lb["mass"] = 1.0
        lb["local_inertia"] = box_inertia(1.0, (0.15, 0.45, 0.15))
        pos = np.zeros((chains * links, 3), F)
        for c in range(chains):
            x0, z0 = (c % side - (side - 1) / 2.0) * spacing, (c // side - (side - 1) / 2.0) * spacing
            v = rng.normal(0.0, 2.0, 2)
            for i in range(links):
                k = c * links + i
                pos[k] = (x0, top - 0.5 - 1.0 * i, z0)
                lb["linear_velocity"][k] = (v[0] * (i + 1) / links, 0.0, v[1] * (i + 1) / links)
        lb["transform"][:, 9:] = pos
        fb = _bodies(loose)
        fb["shape"] = 2
        fb["mass"] = 2.0
        fb["local_inertia"] = box_inertia(2.0, (0.3, 0.3, 0.3))
        half = side * spacing / 2.0
        fpos = np.stack([rng.uniform(-half, half, loose), rng.uniform(top + 1.0, top + 6.0, loose),
                         rng.uniform(-half, half, loose)], 1)
        _set_transforms(fb, random_rotations(rng, loose), fpos)
        bodies = np.concatenate([plane, lb, fb])
        first = base + 1
        for c in range(chains):
            x0, y0, z0 = pos[c * links]
            joints.append({"a": first + c * links, "b": -1, "pivot_a": (0.0, 0.5, 0.0),
                           "pivot_b": (float(x0), float(y0 + 0.5), float(z0))})
            for i in range(links - 1):
                joints.append({"a": first + c * links + i, "b": first + c * links + i + 1,
                               "pivot_a": (0.0, -0.5, 0.0), "pivot_b": (0.0, 0.5, 0.0)})
        all_bodies.append(bodies)
        wid.append(np.full(len(bodies), wi, np.int32))
        base += len(bodies)
    bodies = np.concatenate(all_bodies)
    bodies["world"] = np.concatenate(wid)
    kw = {"world_of_body": np.concatenate(wid)} if worlds > 1 else {}
    return Scene("jointed_chains_%dx%d_w%d" % (chains, links, worlds), 1.0 / 60.0, steps,
                 {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10}, shapes, bodies,
                 meta={"seed": seed, "joints": joints}, **kw)


def hinged_chains(chains=6, links=6, loose=16, seed=0, spacing=2.5, top=10.0, steps=240, worlds=1):
    """Chains of boxes (half-extents 0.15 x 0.45 x 0.15) joined end to end by hinges, the top
    link hinged to the fixed body (by pivot and axis for c even, by frame for c odd); chain c
    swings about z (c even) or x (c odd), the inner hinges of chains with c % 3 == 1 carry limits
    of +-0.6 rad, chains with c % 3 == 2 drive their top hinge with a motor.  Per world also a door (a 0.5 x 1.0 x 0.05 box) hinged to the fixed body by frame with
    a motor, and two loose boxes held to the same orientation by an angular-only hinge.  Frames
    come from the reference's constructors (jbgpu.frames).  meta["joints"]: type "hinge",
    a, b, frame_a, frame_b, optional limit / motor / angular_only."""
    from .frames import hinge_frames_two_bodies, hinge_frames_one_body, hinge_frames_from_frames
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE), {"type": _abi.SHAPE_BOX, "params": (0.15, 0.45, 0.15, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.3, 0.3, 0.3, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.5, 1.0, 0.05, 0.0), "points": None}]
    side = int(np.ceil(np.sqrt(chains)))
    all_bodies, joints, wid = [], [], []
    base = 0
    eye = np.eye(3, dtype=F)
    for wi in range(worlds):
        plane = _plane_body(0)
        lb = _bodies(chains * links)
        lb["shape"] = 1
        lb["mass"] = 1.0
        lb["local_inertia"] = box_inertia(1.0, (0.15, 0.45, 0.15))
        pos = np.zeros((chains * links, 3), F)
        for c in range(chains):
            x0, z0 = (c % side - (side - 1) / 2.0) * spacing, (c // side - (side - 1) / 2.0) * spacing
            v = rng.normal(0.0, 2.0)
            for i in range(links):
                k = c * links + i
                pos[k] = (x0, top - 0.5 - 1.0 * i, z0)
                lin = (0.0, 0.0, v * (i + 1) / links) if c % 2 else (v * (i + 1) / links, 0.0, 0.0)
                lb["linear_velocity"][k] = lin
        lb["transform"][:, 9:] = pos
        door = _bodies(1)
        door["shape"] = 3
        door["mass"] = 2.0
        door["local_inertia"] = box_inertia(2.0, (0.5, 1.0, 0.05))
        half = side * spacing / 2.0
        door["transform"][0, 9:] = (half + 2.0, 1.5, 0.0)
        fb = _bodies(loose)
        fb["shape"] = 2
        fb["mass"] = 2.0
        fb["local_inertia"] = box_inertia(2.0, (0.3, 0.3, 0.3))
        fpos = np.stack([rng.uniform(-half, half, loose), rng.uniform(top + 1.0, top + 6.0, loose),
                         rng.uniform(-half, half, loose)], 1)
        _set_transforms(fb, random_rotations(rng, loose), fpos)
        bodies = np.concatenate([plane, lb, door, fb])
        first = base + 1
        for c in range(chains):
            axis = (1.0, 0.0, 0.0) if c % 2 else (0.0, 0.0, 1.0)
            a0 = first + c * links
            if c % 2:   # by frame: z along x (the pivot/axis form degenerates for an axis along x)
                top_frame = np.concatenate([np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]], F).reshape(9), [0.0, 0.5, 0.0]])
                fa, fb_ = hinge_frames_from_frames(lb["transform"][c * links], top_frame)
            else:
                fa, fb_ = hinge_frames_one_body(lb["transform"][c * links], (0.0, 0.5, 0.0), axis)
            j = {"type": "hinge", "a": a0, "b": -1, "frame_a": fa, "frame_b": fb_}
            if c % 3 == 2:
                j["motor"] = (True, 1.5, 0.05)
            joints.append(j)
            for i in range(links - 1):
                fa, fb_ = hinge_frames_two_bodies(eye, (0.0, -0.5, 0.0), (0.0, 0.5, 0.0), axis, axis)
                j = {"type": "hinge", "a": a0 + i, "b": a0 + i + 1, "frame_a": fa, "frame_b": fb_}
                if c % 3 == 1:
                    j["limit"] = (-0.6, 0.6, 0.9, 0.3, 1.0)
                joints.append(j)
        di = first + chains * links
        door_frame = np.concatenate([np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], F).reshape(9), [-0.5, 0.0, 0.0]])
        fa, fb_ = hinge_frames_from_frames(door["transform"][0], door_frame)
        joints.append({"type": "hinge", "a": di, "b": -1, "frame_a": fa, "frame_b": fb_, "motor": (True, -2.0, 5.0)})
        if loose >= 2:
            fa, fb_ = hinge_frames_two_bodies(fb["transform"][0, :9], (0.0, 0.0, 0.0), (0.0, 0.0, 0.0),
                                              (0.0, 1.0, 0.0), (0.0, 1.0, 0.0))
            joints.append({"type": "hinge", "a": di + 1, "b": di + 2, "frame_a": fa, "frame_b": fb_,
                           "angular_only": True})
        all_bodies.append(bodies)
        wid.append(np.full(len(bodies), wi, np.int32))
        base += len(bodies)
    bodies = np.concatenate(all_bodies)
    bodies["world"] = np.concatenate(wid)
    kw = {"world_of_body": np.concatenate(wid)} if worlds > 1 else {}
    return Scene("hinged_chains_%dx%d_w%d" % (chains, links, worlds), 1.0 / 60.0, steps,
                 {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10}, shapes, bodies,
                 meta={"seed": seed, "joints": joints}, **kw)


def sixdof_chains(chains=4, links=5, loose=8, seed=0, spacing=2.5, top=10.0, steps=240, worlds=1):
    """Chains of boxes (half-extents 0.15 x 0.45 x 0.15) joined end to end by generic 6-dof joints,
    the top link jointed to a static anchor box.  Per chain c: c % 4 == 0 angular limits of
    +-0.4 rad on all three axes; 1 rotation about x only (the other two angular axes locked);
    2 a linear axis free within +-0.3, softer linear rows, a motor on angular axis 0 and limits on
    the others; 3 frames of B as the linear reference, limits with bounce and a motor on axis 2.
    Loose boxes fall on them.  meta["joints"]: type "6dof", a, b, frame_a, frame_b, use_a, limits
    [(axis, lo, hi)], optional linear_motor, angular_motors."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE), {"type": _abi.SHAPE_BOX, "params": (0.15, 0.45, 0.15, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.3, 0.3, 0.3, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.2, 0.2, 0.2, 0.0), "points": None}]
    side = int(np.ceil(np.sqrt(chains)))
    ident = np.eye(3, dtype=F).reshape(9)

    def frame(origin):
        return np.concatenate([ident, np.asarray(origin, F)]).astype(F)
    all_bodies, joints, wid = [], [], []
    base = 0
    for wi in range(worlds):
        plane = _plane_body(0)
        anchors = _bodies(chains)
        anchors["shape"] = 3
        lb = _bodies(chains * links)
        lb["shape"] = 1
        lb["mass"] = 1.0
        lb["local_inertia"] = box_inertia(1.0, (0.15, 0.45, 0.15))
        for c in range(chains):
            x0, z0 = (c % side - (side - 1) / 2.0) * spacing, (c // side - (side - 1) / 2.0) * spacing
            anchors["transform"][c, 9:] = (x0, top + 0.2, z0)
            v = rng.normal(0.0, 1.5, 2)
            for i in range(links):
                k = c * links + i
                lb["transform"][k, 9:] = (x0, top - 0.5 - 1.0 * i, z0)
                lb["linear_velocity"][k] = (v[0] * (i + 1) / links, 0.0, v[1] * (i + 1) / links)
        half = side * spacing / 2.0
        fb = _bodies(loose)
        fb["shape"] = 2
        fb["mass"] = 2.0
        fb["local_inertia"] = box_inertia(2.0, (0.3, 0.3, 0.3))
        fpos = np.stack([rng.uniform(-half, half, loose), rng.uniform(top + 1.0, top + 6.0, loose),
                         rng.uniform(-half, half, loose)], 1)
        _set_transforms(fb, random_rotations(rng, loose), fpos)
        bodies = np.concatenate([plane, anchors, lb, fb])
        first_anchor, first_link = base + 1, base + 1 + chains
        for c in range(chains):
            kind = c % 4
            cfg = {"type": "6dof", "use_a": kind != 3, "limits": []}
            if kind == 0:
                cfg["limits"] = [(3, -0.4, 0.4), (4, -0.4, 0.4), (5, -0.4, 0.4)]
            elif kind == 1:
                cfg["limits"] = [(3, 1.0, -1.0), (4, 0.0, 0.0), (5, 0.0, 0.0)]
            elif kind == 2:
                cfg["limits"] = [(0, -0.3, 0.3), (4, -0.2, 0.2), (5, -0.2, 0.2)]
                cfg["linear_motor"] = (0.8, 1.0, 0.3)
                cfg["angular_motors"] = [(0, True, 0.5, 0.2)]
            else:
                cfg["limits"] = [(3, -0.3, 0.3), (4, -0.3, 0.3), (5, -0.3, 0.3)]
                cfg["angular_motors"] = [(2, True, -0.5, 1.0, 300.0, 1.0, 0.5, 0.3, 0.2)]
            a0 = first_link + c * links
            joints.append(dict(cfg, a=a0, b=first_anchor + c, frame_a=frame((0.0, 0.5, 0.0)),
                               frame_b=frame((0.0, -0.2, 0.0))))
            for i in range(links - 1):
                joints.append(dict(cfg, a=a0 + i, b=a0 + i + 1, frame_a=frame((0.0, -0.5, 0.0)),
                                   frame_b=frame((0.0, 0.5, 0.0))))
        all_bodies.append(bodies)
        wid.append(np.full(len(bodies), wi, np.int32))
        base += len(bodies)
    bodies = np.concatenate(all_bodies)
    bodies["world"] = np.concatenate(wid)
    kw = {"world_of_body": np.concatenate(wid)} if worlds > 1 else {}
    return Scene("sixdof_chains_%dx%d_w%d" % (chains, links, worlds), 1.0 / 60.0, steps,
                 {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10}, shapes, bodies,
                 meta={"seed": seed, "joints": joints}, **kw)


def cone_chains(chains=6, links=5, loose=8, seed=0, spacing=2.5, top=10.0, steps=240, worlds=1):
    """Chains of boxes (half-extents 0.15 x 0.45 x 0.15) joined end to end by cone-twist joints
    whose twist axis (frame x) runs down the chain, the top link jointed to a static anchor box.
    Chain c: c % 3 == 0 setLimit(0.5, 0.5, 0.3); 1 setLimit(0.3, 0.6, 0) (twist locked, with
    softness, bias and relaxation given); 2 no limit set (the constructors' spans of 1e30 and
    softness 0).  Loose boxes fall beside the chains; per world two of them are held to the same
    orientation by an angular-only cone twist.  meta["joints"]: type "cone", a, b, frame_a, frame_b, optional limit, angular_only."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE), {"type": _abi.SHAPE_BOX, "params": (0.15, 0.45, 0.15, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.3, 0.3, 0.3, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.2, 0.2, 0.2, 0.0), "points": None}]
    side = int(np.ceil(np.sqrt(chains)))
    basis = np.array([[0, 1, 0], [-1, 0, 0], [0, 0, 1]], F).reshape(9)   # columns: x down the chain

    def frame(origin):
        return np.concatenate([basis, np.asarray(origin, F)]).astype(F)
    all_bodies, joints, wid = [], [], []
    base = 0
    for wi in range(worlds):
        plane = _plane_body(0)
        anchors = _bodies(chains)
        anchors["shape"] = 3
        lb = _bodies(chains * links)
        lb["shape"] = 1
        lb["mass"] = 1.0
        lb["local_inertia"] = box_inertia(1.0, (0.15, 0.45, 0.15))
        for c in range(chains):
            x0, z0 = (c % side - (side - 1) / 2.0) * spacing, (c // side - (side - 1) / 2.0) * spacing
            anchors["transform"][c, 9:] = (x0, top + 0.2, z0)
            v = rng.normal(0.0, 1.5, 2)
            w = rng.normal(0.0, 1.0)
            for i in range(links):
                k = c * links + i
                lb["transform"][k, 9:] = (x0, top - 0.5 - 1.0 * i, z0)
                lb["linear_velocity"][k] = (v[0] * (i + 1) / links, 0.0, v[1] * (i + 1) / links)
                lb["angular_velocity"][k] = (0.0, w, 0.0)
        half = side * spacing / 2.0
        fb = _bodies(loose)
        fb["shape"] = 2
        fb["mass"] = 2.0
        fb["local_inertia"] = box_inertia(2.0, (0.3, 0.3, 0.3))
        fpos = np.stack([rng.uniform(half + 1.0, half + 4.0, loose), rng.uniform(1.0, 6.0, loose),
                         rng.uniform(-half, half, loose)], 1)   # beside the chains: impacts of 2 kg boxes
                                                                 # drive the 0.5-rad cones unstable
        _set_transforms(fb, random_rotations(rng, loose), fpos)
        bodies = np.concatenate([plane, anchors, lb, fb])
        first_anchor, first_link = base + 1, base + 1 + chains
        for c in range(chains):
            cfg = {"type": "cone"}
            if c % 3 == 0:
                cfg["limit"] = (0.5, 0.5, 0.3, 0.8, 0.3, 1.0)
            elif c % 3 == 1:
                cfg["limit"] = (0.3, 0.6, 0.0, 0.9, 0.4, 0.9)
            a0 = first_link + c * links
            joints.append(dict(cfg, a=a0, b=first_anchor + c, frame_a=frame((0.0, 0.5, 0.0)),
                               frame_b=frame((0.0, -0.2, 0.0))))
            for i in range(links - 1):
                joints.append(dict(cfg, a=a0 + i, b=a0 + i + 1, frame_a=frame((0.0, -0.5, 0.0)),
                                   frame_b=frame((0.0, 0.5, 0.0))))
        if loose >= 2:
            fl = first_link + chains * links
            ra, rb = fb["transform"][0, :9].reshape(3, 3), fb["transform"][1, :9].reshape(3, 3)
            fa_ = np.concatenate([np.eye(3, dtype=F).reshape(9), [0, 0, 0]]).astype(F)
            fb_ = np.concatenate([(rb.T @ ra).astype(F).reshape(9), [0, 0, 0]]).astype(F)
            joints.append({"type": "cone", "a": fl, "b": fl + 1, "frame_a": fa_, "frame_b": fb_,
                           "limit": (0.2, 0.2, 0.2, 0.8, 0.3, 1.0), "angular_only": True})
        all_bodies.append(bodies)
        wid.append(np.full(len(bodies), wi, np.int32))
        base += len(bodies)
    bodies = np.concatenate(all_bodies)
    bodies["world"] = np.concatenate(wid)
    kw = {"world_of_body": np.concatenate(wid)} if worlds > 1 else {}
    return Scene("cone_chains_%dx%d_w%d" % (chains, links, worlds), 1.0 / 60.0, steps,
                 {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10}, shapes, bodies,
                 meta={"seed": seed, "joints": joints}, **kw)


def slider_rigs(rigs=6, loose=8, seed=0, spacing=2.5, steps=240, worlds=1):
    """Boxes (half 0.3, mass 1) on slider joints to static rails (half 1.2 x 0.05 x 0.05) one
    metre above them, sliding along the rail's x.  Rig r: r % 3 == 0 linear limits [-1, 1],
    rotation locked (the defaults' angular limits 0, 0); 1 a powered linear motor and a powered
    angular motor, linear limits [-1.5, 1.5], rotation about the axis free; 2 a vertical rail,
    useLinearReferenceFrameA false with the box as body A, default parameters (free along the
    rail).  Loose boxes fall beside the rigs.  meta["joints"]: type "slider", a, b, frame_a,
    frame_b, use_a, optional params (28 floats, jbgpu_world_set_slider_params order)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE), {"type": _abi.SHAPE_BOX, "params": (0.3, 0.3, 0.3, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (1.2, 0.05, 0.05, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.05, 1.2, 0.05, 0.0), "points": None}]
    defaults = [1.0, -1.0, 0.0, 0.0, 1.0, 0.7, 0.0, 1.0, 0.7, 0.0, 1.0, 0.7, 1.0, 1.0, 0.7, 1.0, 1.0, 0.7, 1.0,
                1.0, 0.7, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
    side = int(np.ceil(np.sqrt(rigs)))
    ident = np.eye(3, dtype=F).reshape(9)
    vert = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], F).reshape(9)    # columns: x up
    all_bodies, joints, wid = [], [], []
    base = 0
    for wi in range(worlds):
        plane = _plane_body(0)
        rails = _bodies(rigs)
        boxes = _bodies(rigs)
        boxes["shape"] = 1
        boxes["mass"] = 1.0
        boxes["local_inertia"] = box_inertia(1.0, (0.3, 0.3, 0.3))
        for r in range(rigs):
            x0, z0 = (r % side - (side - 1) / 2.0) * spacing, (r // side - (side - 1) / 2.0) * spacing
            if r % 3 == 2:
                rails["shape"][r] = 3
                rails["transform"][r, 9:] = (x0 + 0.5, 3.0, z0)
                boxes["transform"][r, 9:] = (x0, 3.5, z0)
                boxes["linear_velocity"][r] = (0.0, rng.normal(0.0, 1.0), 0.0)
            else:
                rails["shape"][r] = 2
                rails["transform"][r, 9:] = (x0, 4.0, z0)
                boxes["transform"][r, 9:] = (x0, 3.0, z0)
                boxes["linear_velocity"][r] = (rng.normal(0.0, 2.0), 0.0, 0.0)
        half = side * spacing / 2.0
        fb = _bodies(loose)
        fb["shape"] = 1
        fb["mass"] = 1.0
        fb["local_inertia"] = box_inertia(1.0, (0.3, 0.3, 0.3))
        fpos = np.stack([rng.uniform(half + 1.0, half + 4.0, loose), rng.uniform(1.0, 6.0, loose),
                         rng.uniform(-half, half, loose)], 1)
        _set_transforms(fb, random_rotations(rng, loose), fpos)
        bodies = np.concatenate([plane, rails, boxes, fb])
        fr, fx = base + 1, base + 1 + rigs
        for r in range(rigs):
            if r % 3 == 2:
                joints.append({"type": "slider", "a": fx + r, "b": fr + r, "use_a": False,
                               "frame_a": np.concatenate([vert, [0.0, 0.0, 0.0]]).astype(F),
                               "frame_b": np.concatenate([vert, [-0.5, 0.0, 0.0]]).astype(F)})
                continue
            p = list(defaults)
            if r % 3 == 0:
                p[0], p[1] = -1.0, 1.0
            else:
                p[0], p[1], p[2], p[3] = -1.5, 1.5, 1.0, -1.0
                p[22], p[23], p[24] = 1.0, 1.0, 5.0
                p[25], p[26], p[27] = 1.0, 2.0, 3.0
            joints.append({"type": "slider", "a": fr + r, "b": fx + r, "use_a": True,
                           "frame_a": np.concatenate([ident, [0.0, -1.0, 0.0]]).astype(F),
                           "frame_b": np.concatenate([ident, [0.0, 0.0, 0.0]]).astype(F), "params": p})
        all_bodies.append(bodies)
        wid.append(np.full(len(bodies), wi, np.int32))
        base += len(bodies)
    bodies = np.concatenate(all_bodies)
    bodies["world"] = np.concatenate(wid)
    kw = {"world_of_body": np.concatenate(wid)} if worlds > 1 else {}
    return Scene("slider_rigs_%d_w%d" % (rigs, worlds), 1.0 / 60.0, steps,
                 {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10}, shapes, bodies,
                 meta={"seed": seed, "joints": joints}, **kw)


def small_mixed(n=60, seed=0, region=(6.0, 8.0, 6.0), steps=200, with_hulls=True):
    """A small dense mix of every shape type for stage-by-stage parity checks."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE)]
    b = _bodies(n)
    for i in range(n):
        k = i % (4 if with_hulls else 3)
        if k == 0:
            r = F(rng.uniform(0.2, 0.6))
            shapes.append({"type": _abi.SHAPE_SPHERE, "params": (float(r), 0, 0, 0), "points": None})
            m = F(1.0); b["local_inertia"][i] = sphere_inertia(m, r)
        elif k == 1:
            h = rng.uniform(0.2, 0.6, 3).astype(F)
            shapes.append({"type": _abi.SHAPE_BOX, "params": (float(h[0]), float(h[1]), float(h[2]), 0), "points": None})
            m = F(1.0); b["local_inertia"][i] = box_inertia(m, h)
        elif k == 2:
            height = F(2.0 * rng.uniform(0.2, 0.8))
            shapes.append({"type": _abi.SHAPE_CAPSULE, "params": (0.25, float(height), 0, 0), "points": None})
            m = F(1.0); b["local_inertia"][i] = capsule_inertia(m, F(0.25), height)
        else:
            d = rng.standard_normal((32, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True)
            pts = (d * rng.uniform(0.3, 1.0, 3)).astype(F)
            shapes.append({"type": _abi.SHAPE_CONVEX_HULL, "params": (0, 0, 0, 0), "points": pts})
            m = F(1.0); b["local_inertia"][i] = hull_inertia(m, pts)
        b["mass"][i] = m
        b["shape"][i] = i + 1
    pos = np.stack([rng.uniform(-region[0] / 2, region[0] / 2, n), rng.uniform(0.5, 0.5 + region[1], n),
                    rng.uniform(-region[2] / 2, region[2] / 2, n)], 1)
    _set_transforms(b, random_rotations(rng, n), pos)
    b["linear_velocity"] = rng.standard_normal((n, 3)).astype(F)
    bodies = np.concatenate([_plane_body(0), b])
    return Scene("small_mixed_%d" % n, 1.0 / 60.0, steps, {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10},
                 shapes, bodies, meta={"seed": seed})


def learned_warmstart(n=100_000, seed=0, pyramids=50, levels=15, region=(200.0, 100.0, 200.0), steps=600):
    """The learned-warm-start workload: the 100k mixed bodies plus `pyramids` 2-D pyramids of
    `levels` levels of unit boxes (half-extent 0.5, mass 1, 120 boxes for 15 levels) standing on
    the plane at seeded, non-overlapping places inside the region (a solver-hard case)."""
    base = mixed_100k(n, seed=seed, region=region, steps=steps) if n > 0 else None
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    per = levels * (levels + 1) // 2
    shapes = list(base.shapes) if base is not None else [dict(PLANE)]
    box_id = len(shapes)
    shapes.append({"type": _abi.SHAPE_BOX, "params": (0.5, 0.5, 0.5, 0.0), "points": None})
    b = _bodies(pyramids * per)
    b["shape"] = box_id
    b["mass"] = 1.0
    b["local_inertia"] = box_inertia(F(1.0), (0.5, 0.5, 0.5))
    centres = []
    span = float(levels) + 2.0
    while len(centres) < pyramids:
        c = rng.uniform(-region[0] / 2 + span, region[0] / 2 - span, 2)
        if all(abs(c[0] - d[0]) > span or abs(c[1] - d[1]) > 3.0 for d in centres):
            centres.append(c)
    pos = []
    for c in centres:
        for lv in range(levels):
            for k in range(levels - lv):
                pos.append((c[0] + (k - (levels - lv - 1) / 2.0), 0.5 + lv, c[1]))
    b["transform"][:, 9:] = np.array(pos, F)
    if base is None:
        bodies = np.concatenate([_plane_body(0), b])
        cfg = {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10}
        dt = 1.0 / 120.0
    else:
        bodies = np.concatenate([base.bodies, b])
        cfg, dt = base.config, base.dt
    return Scene("learned_warmstart_%d_%dx%d" % (n, pyramids, levels), dt, steps, cfg, shapes, bodies,
                 meta={"seed": seed, "pyramid_bodies": pyramids * per})


def ccd_shots(shots=24, seed=0, steps=90, plane=False, threshold=0.05, swept_radius=0.08):
    """Fast projectiles fired at thin walls, for CCD motion clamping (DiscreteDynamicsWorld.
    integrateTransforms' CCD branch): a static box floor (no static plane, since the reference's
    CCD sweep throws on one), two thin static walls across the x axis, a few loose dynamic boxes
    in front of them, and `shots` small spheres and boxes moving at 50-90 m/s along +x (about a
    metre per 1/60 s step, ten times the walls' thickness), some in pairs on one path.  The shots
    get the CCD motion threshold and swept-sphere radius in meta["ccd"]; plane=True puts a static
    plane in the world first (the reference throws when a sweep reaches it)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [{"type": _abi.SHAPE_BOX, "params": (30.0, 0.5, 30.0, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.05, 2.5, 4.0, 0.0), "points": None},
              {"type": _abi.SHAPE_SPHERE, "params": (0.1, 0.0, 0.0, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.1, 0.1, 0.1, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.4, 0.4, 0.4, 0.0), "points": None}]
    parts = []
    if plane:
        shapes.append(dict(PLANE))
        parts.append(_plane_body(len(shapes) - 1))
    fixed = _bodies(3)
    fixed["shape"] = [0, 1, 1]
    fixed["transform"][:, 9:] = np.array([[0.0, -0.5, 0.0], [6.0, 2.5, 0.0], [12.0, 2.5, 0.0]], F)
    parts.append(fixed)
    loose = _bodies(6)
    loose["shape"] = 4
    loose["mass"] = 2.0
    loose["local_inertia"] = box_inertia(2.0, (0.4, 0.4, 0.4))
    loose["transform"][:, 9:] = np.stack([np.repeat([5.2, 11.2], 3), np.full(6, 0.41),
                                          np.tile([-2.0, 0.0, 2.0], 2)], 1).astype(F)
    parts.append(loose)
    shots_b = _bodies(shots)
    kind = rng.integers(0, 2, shots)
    shots_b["shape"] = np.where(kind == 0, 2, 3)
    shots_b["mass"] = 0.1
    shots_b["local_inertia"] = np.where((kind == 0)[:, None], sphere_inertia(0.1, 0.1), box_inertia(0.1, (0.1, 0.1, 0.1)))
    pos = np.stack([rng.uniform(-1.0, 2.0, shots), rng.uniform(0.4, 4.0, shots), rng.uniform(-3.0, 3.0, shots)], 1)
    for k in range(1, shots, 4):          # every fourth shot follows another on its path
        pos[k] = pos[k - 1] - np.array([0.6, 0.0, 0.0])
    _set_transforms(shots_b, random_rotations(rng, shots), pos)
    vel = np.stack([rng.uniform(50.0, 90.0, shots), rng.uniform(-2.0, 2.0, shots), rng.uniform(-3.0, 3.0, shots)], 1)
    for k in range(1, shots, 4):
        vel[k] = vel[k - 1]
    shots_b["linear_velocity"] = vel.astype(F)
    shots_b["angular_velocity"] = rng.uniform(-20.0, 20.0, (shots, 3)).astype(F)
    parts.append(shots_b)
    bodies = np.concatenate(parts)
    first = len(bodies) - shots
    return Scene("ccd_shots_%d%s" % (shots, "_plane" if plane else ""), 1.0 / 60.0, steps,
                 {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10}, shapes, bodies,
                 meta={"seed": seed, "ccd": {"bodies": list(range(first, len(bodies))), "threshold": threshold,
                                             "radius": swept_radius}, "walls_x": (6.0, 12.0)})


# ---- kinematic and trigger bodies ------------------------------------------------------------
def kinematic_platforms(platforms=4, boxes=3, seed=0, steps=240):
    """Kinematic platforms (mass 0, KINEMATIC_OBJECT, DISABLE_DEACTIVATION) that the caller moves
    every step (kinematic_pose) along small loops with a slow turn about y, dynamic boxes dropped
    onto them, a ground plane; a static trigger box (NO_CONTACT_RESPONSE) under a box that falls
    through it, a trigger sphere (dynamic, NO_CONTACT_RESPONSE) that falls through the ground, and
    a kinematic box left at rest with the default activation (it falls asleep)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE),
              {"type": _abi.SHAPE_BOX, "params": (1.5, 0.2, 1.5, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (0.3, 0.3, 0.3, 0.0), "points": None},
              {"type": _abi.SHAPE_BOX, "params": (1.0, 0.5, 1.0, 0.0), "points": None},
              {"type": _abi.SHAPE_SPHERE, "params": (0.4, 0.0, 0.0, 0.0), "points": None}]
    parts = [_plane_body(0)]
    base = np.array([[6.0 * (k % 2) - 3.0, 2.0 + 0.5 * (k // 2), 6.0 * (k // 2) - 3.0] for k in range(platforms)])
    kin = _bodies(platforms)
    kin["shape"] = 1
    kin["collision_flags"] = _abi.CF_KINEMATIC_OBJECT
    kin["activation_state"] = _abi.DISABLE_DEACTIVATION
    kin["transform"][:, [0, 4, 8]] = 1.0
    kin["transform"][:, 9:] = base.astype(F)
    parts.append(kin)
    box = _bodies(platforms * boxes)
    box["shape"] = 2
    box["mass"] = 1.0
    box["local_inertia"] = box_inertia(1.0, (0.3, 0.3, 0.3))
    pos = np.repeat(base, boxes, 0) + np.stack([rng.uniform(-0.8, 0.8, platforms * boxes),
                                                np.tile(0.8 + 0.7 * np.arange(boxes), platforms),
                                                rng.uniform(-0.8, 0.8, platforms * boxes)], 1)
    _set_transforms(box, random_rotations(rng, platforms * boxes), pos)
    parts.append(box)
    extra = _bodies(4)
    extra["shape"] = [3, 2, 4, 2]
    extra["mass"] = [0.0, 1.0, 2.0, 0.0]
    extra["collision_flags"] = [_abi.CF_NO_CONTACT_RESPONSE, 0, _abi.CF_NO_CONTACT_RESPONSE, _abi.CF_KINEMATIC_OBJECT]
    extra["local_inertia"][1] = box_inertia(1.0, (0.3, 0.3, 0.3))
    extra["local_inertia"][2] = sphere_inertia(2.0, 0.4)
    extra["transform"][:, [0, 4, 8]] = 1.0
    extra["transform"][:, 9:] = np.array([[10.0, 0.5, 0.0], [10.0, 2.5, 0.0], [-10.0, 3.0, 0.0], [0.0, 0.3, 10.0]], F)
    parts.append(extra)
    bodies = np.concatenate(parts)
    return Scene("kinematic_platforms_%d" % platforms, 1.0 / 60.0, steps, {"gravity": (0.0, -9.81, 0.0)}, shapes,
                 bodies, meta={"seed": seed, "kinematic": {"bodies": list(range(1, 1 + platforms)), "base": base}})


def kinematic_pose(scene, step):
    """The poses of the moving kinematic platforms at `step` (12 binary32 values each): origins
    on loops of 1.2 m radius at about 1 m/s (faster than the sleeping threshold), turned about y
    by up to 0.3 rad."""
    k = scene.meta["kinematic"]
    t = step * scene.dt
    out = np.zeros((len(k["bodies"]), 12), F)
    for j, base in enumerate(k["base"]):
        ph = 0.7 * j
        a = 0.3 * np.sin(0.5 * t + ph)
        c, s = np.cos(a), np.sin(a)
        out[j, :9] = np.array([c, 0.0, s, 0.0, 1.0, 0.0, -s, 0.0, c], F)
        out[j, 9:] = (base + np.array([1.2 * np.sin(0.8 * t + ph), 0.2 * np.sin(1.1 * t + ph),
                                       1.2 * np.cos(0.8 * t + ph) - 1.2])).astype(F)
    return out


# ---- compound and concave shapes ----------------------------------------------------------
def _f(x):
    return F(x)


def _row_dot(b, r, v):
    """dot(row r of the 3x3 `b`, v) in binary32, x*x' + y*y' + z*z' in that order."""
    return F(F(F(b[r, 0] * v[0]) + F(b[r, 1] * v[1])) + F(b[r, 2] * v[2]))


def _xf_apply(b, o, v):
    """Transform.transform: v.mul(basis) (rows dotted with v) plus the origin, binary32."""
    return np.array([F(_row_dot(b, r, v) + o[r]) for r in range(3)], F)


def convex_aabb(shape, xf12):
    """CollisionShape.getAabb of a box, sphere, capsule or hull at a transform, binary32 in the
    reference's operation order (BoxShape.java:146-151 via AabbUtil2.transformAabb,
    SphereShape.java:56-65, CapsuleShape.java:160-190, PolyhedralConvexShape.java:163-171)."""
    t = np.asarray(xf12, F)
    b, o = t[:9].reshape(3, 3), t[9:12]
    ab = np.abs(b)
    m = F(0.04)
    k = shape["type"]
    if k == _abi.SHAPE_SPHERE:
        r = F(shape["params"][0])
        e = np.array([r, r, r], F)
        return o - e, o + e
    if k == _abi.SHAPE_BOX:
        he = np.array(shape["params"][:3], F)
        dims = he * F(1) - m
        hem = dims + m
        c = o
    elif k == _abi.SHAPE_CAPSULE:
        r, hh = F(shape["params"][0]), F(F(0.5) * F(shape["params"][1]))
        hem = np.array([r, F(r + hh), r], F) + m
        c = o
    elif k == _abi.SHAPE_CONVEX_HULL:
        mn, mx = hull_local_aabb(shape["points"], m)
        hem = (mx - mn) * F(0.5) + m
        c = _xf_apply(b, o, (mx + mn) * F(0.5))
    else:
        raise ValueError("not a convex shape on this path")
    e = np.array([_row_dot(ab, r, hem) for r in range(3)], F)
    return c - e, c + e


def compound_local_aabb(children):
    """CompoundShape.addChildShape's running union (CompoundShape.java:59-91)."""
    mn = np.full(3, 1e30, F)
    mx = np.full(3, -1e30, F)
    for shape, xf in children:
        a, b = convex_aabb(shape, xf)
        mn, mx = np.minimum(mn, a), np.maximum(mx, b)
    return mn, mx


def compound_inertia(mass, children, margin=0.0):
    """CompoundShape.calculateLocalInertia: the box inertia of getAabb(identity)
    (CompoundShape.java:222-243 and 126-171)."""
    mn, mx = compound_local_aabb(children)
    lhe = (mx - mn) * F(0.5) + F(margin)
    lc = (mx + mn) * F(0.5)
    amin, amax = lc - lhe, lc + lhe
    he = (amax - amin) * F(0.5)
    lx, ly, lz = F(2) * he[0], F(2) * he[1], F(2) * he[2]
    m12 = F(F(mass) / F(12))
    return np.array([m12 * (ly * ly + lz * lz), m12 * (lx * lx + lz * lz), m12 * (lx * lx + ly * ly)], F)


def xf12(basis=None, origin=(0.0, 0.0, 0.0)):
    b = np.eye(3, dtype=F) if basis is None else np.asarray(basis, F).reshape(3, 3)
    return np.concatenate([b.reshape(9), np.asarray(origin, F)]).astype(F)


def rot_x(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]], F)


def rot_z(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], F)


def terrain_mesh(nx=24, nz=24, size=24.0, amp=1.2, seed=0, margin=0.0, bowl=0.4, scaling=(0.0, 0.0, 0.0)):
    """A heightfield of nx x nz cells over size x size m (two triangles per cell, alternating
    diagonals, counter-clockwise seen from above) with smooth random bumps of about amp m on a
    bowl: the shape dict of a BvhTriangleMeshShape (scaling: its setLocalScaling, (0, 0, 0) none)."""
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    xs = np.linspace(-size / 2, size / 2, nx + 1)
    zs = np.linspace(-size / 2, size / 2, nz + 1)
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    H = np.zeros_like(X)
    for _ in range(6):
        kx, kz, ph = rng.uniform(0.1, 0.5), rng.uniform(0.1, 0.5), rng.uniform(0, 2 * np.pi)
        H += amp / 3 * np.sin(kx * X + ph) * np.cos(kz * Z - ph)
    H += rng.uniform(-0.05, 0.05, H.shape)
    H += bowl * (X * X + Z * Z) / size     # a bowl (edges bowl * size / 2 higher), so that what lands stays on it
    verts = np.stack([X, H, Z], -1).reshape(-1, 3).astype(F)
    idx = []
    for i in range(nx):
        for j in range(nz):
            a, b, c, d = i * (nz + 1) + j, (i + 1) * (nz + 1) + j, (i + 1) * (nz + 1) + j + 1, i * (nz + 1) + j + 1
            if (i + j) % 2 == 0:
                idx += [(a, d, c), (a, c, b)]
            else:
                idx += [(a, d, b), (d, c, b)]
    return {"type": _abi.SHAPE_TRIANGLE_MESH, "params": (float(margin),) + tuple(float(x) for x in scaling),
            "points": verts, "indices": np.asarray(idx, np.int32)}


def _convex_kinds(rng, n, hull_pts=12):
    """n random convex shape dicts (boxes, spheres, capsules, hulls) with their masses (density 1000)."""
    out = []
    for i in range(n):
        k = i % 4
        if k == 0:
            h = rng.uniform(0.2, 0.5, 3).astype(F)
            s = {"type": _abi.SHAPE_BOX, "params": (float(h[0]), float(h[1]), float(h[2]), 0.0), "points": None}
            m = F(1000.0 * 8.0 * float(h[0]) * float(h[1]) * float(h[2]))
            inertia = box_inertia(m, h)
        elif k == 1:
            r = F(rng.uniform(0.2, 0.5))
            s = {"type": _abi.SHAPE_SPHERE, "params": (float(r), 0.0, 0.0, 0.0), "points": None}
            m = F(1000.0 * 4.0 / 3.0 * np.pi * float(r) ** 3)
            inertia = sphere_inertia(m, r)
        elif k == 2:
            r, height = F(0.2), F(rng.uniform(0.4, 1.2))
            s = {"type": _abi.SHAPE_CAPSULE, "params": (float(r), float(height), 0.0, 0.0), "points": None}
            m = F(1000.0 * (np.pi * 0.04 * float(height) + 4.0 / 3.0 * np.pi * 0.008))
            inertia = capsule_inertia(m, r, height)
        else:
            ax = rng.uniform(0.25, 0.5, 3)
            d = rng.standard_normal((hull_pts, 3))
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            pts = (d * ax).astype(F)
            s = {"type": _abi.SHAPE_CONVEX_HULL, "params": (0.0, 0.0, 0.0, 0.0), "points": pts}
            m = F(1000.0 * 4.0 / 3.0 * np.pi * ax.prod())
            inertia = hull_inertia(m, pts)
        out.append((s, m, inertia))
    return out


def _compound_kinds(rng, n):
    """n random compound shape dicts with masses: dumbbells (two spheres on a capsule), L shapes
    (two boxes), tables (a top on four legs) and hull pairs, children at rotated transforms."""
    out = []
    for i in range(n):
        k = i % 4
        if k == 0:
            r, L = F(rng.uniform(0.2, 0.35)), F(rng.uniform(0.5, 0.9))
            ch = [({"type": _abi.SHAPE_SPHERE, "params": (float(r), 0.0, 0.0, 0.0), "points": None}, xf12(None, (-L, 0, 0))),
                  ({"type": _abi.SHAPE_SPHERE, "params": (float(r), 0.0, 0.0, 0.0), "points": None}, xf12(None, (L, 0, 0))),
                  ({"type": _abi.SHAPE_CAPSULE, "params": (0.1, float(2 * L), 0.0, 0.0), "points": None},
                   xf12(rot_z(np.pi / 2), (0, 0, 0)))]
            m = F(1000.0 * (2 * 4.0 / 3.0 * np.pi * float(r) ** 3))
        elif k == 1:
            a = rng.uniform(0.3, 0.6)
            ch = [({"type": _abi.SHAPE_BOX, "params": (float(a), 0.15, 0.15, 0.0), "points": None}, xf12(None, (0, 0, 0))),
                  ({"type": _abi.SHAPE_BOX, "params": (0.15, float(a), 0.15, 0.0), "points": None},
                   xf12(rot_x(0.3), (float(a) - 0.15, float(a) - 0.15, 0)))]
            m = F(1000.0 * 2 * 8 * a * 0.15 * 0.15)
        elif k == 2:
            w = rng.uniform(0.5, 0.8)
            ch = [({"type": _abi.SHAPE_BOX, "params": (float(w), 0.06, float(w), 0.0), "points": None}, xf12(None, (0, 0.4, 0)))]
            for sx in (-1, 1):
                for sz in (-1, 1):
                    ch.append(({"type": _abi.SHAPE_BOX, "params": (0.06, 0.2, 0.06, 0.0), "points": None},
                               xf12(None, (sx * (w - 0.1), 0.14, sz * (w - 0.1)))))
            m = F(1000.0 * 8 * w * 0.06 * w)
        else:
            chs = []
            for sgn in (-1, 1):
                d = rng.standard_normal((10, 3))
                d /= np.linalg.norm(d, axis=1, keepdims=True)
                pts = (d * rng.uniform(0.2, 0.4, 3)).astype(F)
                chs.append(({"type": _abi.SHAPE_CONVEX_HULL, "params": (0.0, 0.0, 0.0, 0.0), "points": pts},
                            xf12(rot_z(sgn * 0.4), (sgn * 0.3, 0, 0))))
            ch = chs
            m = F(1000.0 * 0.2)
        s = {"type": _abi.SHAPE_COMPOUND, "params": (0.0, 0.0, 0.0, 0.0), "points": None, "children": ch}
        out.append((s, m, compound_inertia(m, ch)))
    return out


def terrain(n=60, seed=0, cells=16, size=16.0, compounds=0, steps=200, region=(10.0, 6.0, 10.0), y0=4.0, bowl=0.4,
            mesh_scaling=(0.0, 0.0, 0.0)):
    """Convex bodies (boxes, spheres, capsules, hulls; density 1000) and optionally compound bodies
    dropped on a static triangle-mesh terrain (a BvhTriangleMeshShape heightfield of cells x cells
    quads over size x size m, with setLocalScaling(mesh_scaling) unless it is (0, 0, 0)); no plane;
    10 iterations, dt 1/60."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [terrain_mesh(cells, cells, size, seed=seed, bowl=bowl, scaling=mesh_scaling)]
    kinds = _convex_kinds(rng, n) + _compound_kinds(rng, compounds)
    order = rng.permutation(len(kinds))
    kinds = [kinds[i] for i in order]
    nb = len(kinds)
    b = _bodies(nb)
    for i, (s, m, inertia) in enumerate(kinds):
        shapes.append(s)
        b["shape"][i] = i + 1
        b["mass"][i] = m
        b["local_inertia"][i] = inertia
    pos = np.stack([rng.uniform(-region[0] / 2, region[0] / 2, nb), rng.uniform(y0, y0 + region[1], nb),
                    rng.uniform(-region[2] / 2, region[2] / 2, nb)], 1)
    _set_transforms(b, random_rotations(rng, nb), pos)
    ground = _bodies(1)
    ground["shape"] = 0
    bodies = np.concatenate([ground, b])
    return Scene("terrain_%d_c%d" % (n, compounds), 1.0 / 60.0, steps, {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10},
                 shapes, bodies, meta={"seed": seed})


def compounds(n=40, convex=20, seed=0, steps=200, region=(6.0, 10.0, 6.0), y0=1.0):
    """Compound bodies (dumbbells, L shapes, tables, hull pairs; children at rotated transforms)
    and convex bodies dropped on a static plane; 10 iterations, dt 1/60."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shapes = [dict(PLANE)]
    kinds = _compound_kinds(rng, n) + _convex_kinds(rng, convex)
    order = rng.permutation(len(kinds))
    kinds = [kinds[i] for i in order]
    nb = len(kinds)
    b = _bodies(nb)
    for i, (s, m, inertia) in enumerate(kinds):
        shapes.append(s)
        b["shape"][i] = i + 1
        b["mass"][i] = m
        b["local_inertia"][i] = inertia
    pos = np.stack([rng.uniform(-region[0] / 2, region[0] / 2, nb), rng.uniform(y0, y0 + region[1], nb),
                    rng.uniform(-region[2] / 2, region[2] / 2, nb)], 1)
    _set_transforms(b, random_rotations(rng, nb), pos)
    bodies = np.concatenate([_plane_body(0), b])
    return Scene("compounds_%d_%d" % (n, convex), 1.0 / 60.0, steps, {"gravity": (0.0, -9.81, 0.0), "num_iterations": 10},
                 shapes, bodies, meta={"seed": seed})


SCENES = {
    "boxes_1k": boxes_on_plane,
    "mixed_100k": mixed_100k,
    "hulls_20k": hulls,
    "batched_4096": batched_worlds,
    "batched_1024": lambda seed=0: batched_worlds(1024, seed=seed),   # a quarter of it (profiling captures)
    "box_stack": box_stack,
    "small_mixed": small_mixed,
    "learned_warmstart": learned_warmstart,
    "jointed_chains": jointed_chains,
    "hinged_chains": hinged_chains,
    "sixdof_chains": sixdof_chains,
    "cone_chains": cone_chains,
    "slider_rigs": slider_rigs,
    "ccd_shots": ccd_shots,
    "kinematic_platforms": kinematic_platforms,
    "terrain": terrain,
    "compounds": compounds,
    # 20,000 convex and 2,000 compound bodies dropped on a 128 x 128-cell terrain (32,768
    # triangles) over 200 x 200 m
    "terrain_20k": lambda seed=0: terrain(20000, seed=seed, cells=128, size=200.0, compounds=2000, steps=300,
                                          region=(180.0, 40.0, 180.0), y0=6.0, bowl=0.02),
}
