"""ctypes mirror of include/jbgpu.h (the C ABI of the GPU rigid-body step).

The structures here are byte-for-byte the POD structs of the header; both the CUDA
library and the CPU oracle take them, so one set of host buffers feeds either side.
"""
import ctypes as C

import numpy as np

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CAPACITY = 2
ERR_CUDA = 3
ERR_NAN = 4
ERR_TIMEOUT = 5
ERR_UNSUPPORTED = 6
ERR_EPA_OVERFLOW = 7
ERR_NO_DEVICE = 8

SHAPE_BOX = 0
SHAPE_CONVEX_HULL = 4
SHAPE_SPHERE = 6
SHAPE_CAPSULE = 8
SHAPE_TRIANGLE_MESH = 16
SHAPE_STATIC_PLANE = 23
SHAPE_COMPOUND = 25
COMPOUND_MAX_CHILDREN = 16

ACTIVE_TAG = 1
ISLAND_SLEEPING = 2
WANTS_DEACTIVATION = 3
DISABLE_DEACTIVATION = 4
DISABLE_SIMULATION = 5

SOLVER_RANDMIZE_ORDER = 1
SOLVER_FRICTION_SEPARATE = 2
SOLVER_USE_WARMSTARTING = 4
SOLVER_CACHE_FRIENDLY = 8

STAGE_APPLY_GRAVITY = 0
STAGE_PREDICT = 1
STAGE_AABB = 2
STAGE_PAIRS = 3
STAGE_NARROWPHASE = 4
STAGE_ISLANDS = 5
STAGE_SOLVE = 6
STAGE_INTEGRATE = 7
STAGE_ACTIVATION = 8
STAGE_CLEAR_FORCES = 9
STAGE_SAVE_KINEMATIC = 10

CF_STATIC_OBJECT = 1
CF_KINEMATIC_OBJECT = 2
CF_NO_CONTACT_RESPONSE = 4

# per-body properties settable after the bodies were added, in the C call's argument order
BODY_PROPERTIES = ("linear_damping", "angular_damping", "friction", "restitution", "linear_sleeping_threshold",
                   "angular_sleeping_threshold")
# DynamicsWorld.setInternalTickCallback: (world handle, time step, user pointer)
TICK_CALLBACK = C.CFUNCTYPE(None, C.c_void_p, C.c_float, C.c_void_p)


def body_property_arrays(bodies, props):
    """The bodies as int32 and one float32 array per named property (None where not given)."""
    b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
    bad = set(props) - set(BODY_PROPERTIES)
    if bad:
        raise TypeError(f"unknown body properties {sorted(bad)}")
    arrs = [None if props.get(k) is None else
            np.ascontiguousarray(np.broadcast_to(np.asarray(props[k], np.float32).reshape(-1), (len(b),)), np.float32)
            for k in BODY_PROPERTIES]
    return b, arrs


class TickTrampoline:
    """A Python tick callback behind the C function pointer: cb(world, time_step).  An exception in
    it is kept and raised by `reraise` after the stepping call returns (ctypes would swallow it)."""

    def __init__(self, world, cb):
        self.error = None

        def tramp(_h, dt, _user):
            if self.error is not None:
                return
            try:
                cb(world, dt)
            except BaseException as e:   # noqa: BLE001 - kept and raised after the step
                self.error = e
        self.fn = TICK_CALLBACK(tramp)

    def reraise(self):
        if self.error is not None:
            e, self.error = self.error, None
            raise e

POINT_FLOATS = 32
MANIFOLD_POINTS = 4

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)
u64p = C.POINTER(C.c_uint64)


class Config(C.Structure):
    _fields_ = [
        ("gravity", C.c_float * 3),
        ("contact_breaking_threshold", C.c_float),
        ("deactivation_time", C.c_float),
        ("disable_deactivation", C.c_int32),
        ("num_iterations", C.c_int32),
        ("erp", C.c_float),
        ("warmstarting_factor", C.c_float),
        ("linear_slop", C.c_float),
        ("solver_mode", C.c_int32),
        ("device", C.c_int32),
        ("initial_body_capacity", C.c_int32),
        ("pairs_per_body", C.c_int32),
        ("solver_parts", C.c_int32),
        ("solver_threads", C.c_int32),
        ("solver_residual", C.c_float),
        ("solver_max_iterations", C.c_int32),
        ("solver_smem_bodies", C.c_int32),
        ("broadphase_rebuild_interval", C.c_int32),
        ("step_graphs", C.c_int32),
        ("solver_residual_scope", C.c_int32),
    ]


def default_config(**overrides):
    """The reference defaults (ContactSolverInfo, BulletGlobals, DiscreteDynamicsWorld)."""
    c = Config()
    c.gravity[:] = (0.0, -10.0, 0.0)
    c.contact_breaking_threshold = 0.02
    c.deactivation_time = 2.0
    c.disable_deactivation = 0
    c.num_iterations = 10
    c.erp = 0.2
    c.warmstarting_factor = 0.85
    c.linear_slop = 0.0
    c.solver_mode = SOLVER_CACHE_FRIENDLY | SOLVER_USE_WARMSTARTING
    c.device = 0
    c.initial_body_capacity = 1024
    c.pairs_per_body = 16
    c.broadphase_rebuild_interval = 4
    c.step_graphs = 1
    for k, v in overrides.items():
        if k == "gravity":
            c.gravity[:] = tuple(v)
        else:
            setattr(c, k, v)
    return c


class ShapeDesc(C.Structure):
    pass


ShapeDesc._fields_ = [
    ("type", C.c_int32),
    ("params", C.c_float * 4),
    ("points", f32p),
    ("num_points", C.c_int32),
    ("indices", C.POINTER(C.c_int32)),
    ("num_triangles", C.c_int32),
    ("children", C.POINTER(ShapeDesc)),
    ("child_transforms", f32p),
    ("num_children", C.c_int32),
]


class BodyDesc(C.Structure):
    _fields_ = [
        ("mass", C.c_float),
        ("shape", C.c_int32),
        ("transform", C.c_float * 12),
        ("local_inertia", C.c_float * 3),
        ("linear_damping", C.c_float),
        ("angular_damping", C.c_float),
        ("friction", C.c_float),
        ("restitution", C.c_float),
        ("linear_sleeping_threshold", C.c_float),
        ("angular_sleeping_threshold", C.c_float),
        ("linear_velocity", C.c_float * 3),
        ("angular_velocity", C.c_float * 3),
        ("collision_group", C.c_int32),
        ("collision_mask", C.c_int32),
        ("world", C.c_int32),
        ("collision_flags", C.c_int32),
        ("activation_state", C.c_int32),
    ]


class State(C.Structure):
    _fields_ = [
        ("n_bodies", C.c_int32),
        ("transform", f32p),
        ("linear_velocity", f32p),
        ("angular_velocity", f32p),
        ("inv_inertia_world", f32p),
        ("total_force", f32p),
        ("total_torque", f32p),
        ("aabb", f32p),
        ("activation_state", i32p),
        ("deactivation_time", f32p),
        ("island_tag", i32p),
    ]


class Manifolds(C.Structure):
    _fields_ = [
        ("n_pairs", C.c_int32),
        ("capacity", C.c_int32),
        ("keys", u64p),
        ("flags", i32p),
        ("num_points", i32p),
        ("points", f32p),
    ]


class RayHit(C.Structure):
    _fields_ = [
        ("body", C.c_int32),
        ("fraction", C.c_float),
        ("normal", C.c_float * 3),
        ("point", C.c_float * 3),
    ]


RAY_HIT_DTYPE = np.dtype([("body", np.int32), ("fraction", np.float32), ("normal", np.float32, 3),
                          ("point", np.float32, 3)])


class Counters(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("bodies", C.c_int32),
        ("pairs", C.c_int32),
        ("manifolds", C.c_int32),
        ("contacts", C.c_int32),
        ("solver_manifolds", C.c_int32),
        ("solver_rows", C.c_int32),
        ("colours", C.c_int32),
        ("islands", C.c_int32),
        ("gjk_calls", C.c_int32),
        ("epa_calls", C.c_int32),
        ("status_flags", C.c_int32),
        ("solver_iterations", C.c_int32),
        ("cut_colours", C.c_int32),
        ("cut_manifolds", C.c_int32),
        ("solver_islands", C.c_int32),
        ("solver_islands_converged", C.c_int32),
        ("solver_island_iterations", C.c_int32),
        ("ray_replays", C.c_int32),
        ("ccd_clamped", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


STATE_FIELDS = {
    # name: (per-body width, dtype)
    "transform": (12, np.float32),
    "linear_velocity": (3, np.float32),
    "angular_velocity": (3, np.float32),
    "inv_inertia_world": (9, np.float32),
    "total_force": (3, np.float32),
    "total_torque": (3, np.float32),
    "aabb": (6, np.float32),
    "activation_state": (1, np.int32),
    "deactivation_time": (1, np.float32),
    "island_tag": (1, np.int32),
}


class StateBuffers:
    """Host arrays for one body state snapshot plus the ctypes struct pointing at them."""

    def __init__(self, n, fields=None):
        self.n = n
        self.arrays = {}
        for name, (w, dt) in STATE_FIELDS.items():
            if fields is None or name in fields:
                shape = (n,) if w == 1 else (n, w)
                self.arrays[name] = np.zeros(shape, dtype=dt)
        self.struct = State()
        self.struct.n_bodies = n
        for name, (w, dt) in STATE_FIELDS.items():
            a = self.arrays.get(name)
            setattr(self.struct, name, _ptr(a, i32p if dt == np.int32 else f32p))

    @classmethod
    def from_arrays(cls, arrays):
        n = len(next(iter(arrays.values())))
        sb = cls(n, fields=set(arrays.keys()))
        for k, v in arrays.items():
            sb.arrays[k][...] = v
        return sb

    def copy_arrays(self):
        return {k: v.copy() for k, v in self.arrays.items()}


class ManifoldBuffers:
    def __init__(self, capacity):
        self.capacity = capacity
        self.keys = np.zeros(capacity, np.uint64)
        self.flags = np.zeros(capacity, np.int32)
        self.num_points = np.zeros(capacity, np.int32)
        self.points = np.zeros((capacity, MANIFOLD_POINTS, POINT_FLOATS), np.float32)
        self.struct = Manifolds()
        self.struct.capacity = capacity
        self.struct.keys = _ptr(self.keys, u64p)
        self.struct.flags = _ptr(self.flags, i32p)
        self.struct.num_points = _ptr(self.num_points, i32p)
        self.struct.points = _ptr(self.points, f32p)

    @classmethod
    def from_arrays(cls, keys, flags, num_points, points):
        mb = cls(max(1, len(keys)))
        n = len(keys)
        mb.keys[:n] = keys
        mb.flags[:n] = flags
        mb.num_points[:n] = num_points
        mb.points[:n] = points
        mb.struct.n_pairs = n
        return mb

    def view(self):
        n = self.struct.n_pairs
        return {
            "keys": self.keys[:n].copy(),
            "flags": self.flags[:n].copy(),
            "num_points": self.num_points[:n].copy(),
            "points": self.points[:n].copy(),
        }
