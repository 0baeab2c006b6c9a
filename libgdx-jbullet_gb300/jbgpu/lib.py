"""ctypes binding of libjbgpu.so (include/jbgpu.h).

`GpuWorld` is a thin handle over one `jbgpu_world`: scene upload, stepping, stage-by-stage
execution for open-loop checks, and state/manifold snapshots in the host layout of
_abi.StateBuffers / _abi.ManifoldBuffers.  The library is built in-tree (see _build.py);
loading fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import _abi
from ._build import LIB

_lib = None


class JbgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("jbgpu error %d: %s" % (code, msg))
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError("libjbgpu.so is not built (run __graft_entry__.build() or jbgpu._build.build())")
        L = C.CDLL(LIB)
        P = C.POINTER
        sigs = {
            "jbgpu_version": ([], C.c_char_p),
            "jbgpu_launch_count": ([], C.c_int64),
            "jbgpu_last_error": ([], C.c_char_p),
            "jbgpu_config_default": ([P(_abi.Config)], None),
            "jbgpu_shape_local_inertia": ([P(_abi.ShapeDesc), C.c_float, _abi.f32p], C.c_int),
            "jbgpu_shape_mesh_bvh": ([P(_abi.ShapeDesc), _abi.i32p, C.c_int32, _abi.i32p, _abi.f32p], C.c_int),
            "jbgpu_world_create": ([P(_abi.Config), P(C.c_void_p)], C.c_int),
            "jbgpu_world_destroy": ([C.c_void_p], C.c_int),
            "jbgpu_world_add_shape": ([C.c_void_p, P(_abi.ShapeDesc), _abi.i32p], C.c_int),
            "jbgpu_world_add_shapes": ([C.c_void_p, P(_abi.ShapeDesc), C.c_int32, _abi.i32p], C.c_int),
            "jbgpu_world_add_bodies": ([C.c_void_p, P(_abi.BodyDesc), C.c_int32, _abi.i32p], C.c_int),
            "jbgpu_world_num_bodies": ([C.c_void_p, _abi.i32p], C.c_int),
            "jbgpu_world_step_simulation": ([C.c_void_p, C.c_float, C.c_int32, C.c_float, _abi.i32p], C.c_int),
            "jbgpu_world_step": ([C.c_void_p, C.c_float, C.c_int32], C.c_int),
            "jbgpu_world_stage": ([C.c_void_p, C.c_int32, C.c_float], C.c_int),
            "jbgpu_world_synchronize": ([C.c_void_p], C.c_int),
            "jbgpu_world_get_state": ([C.c_void_p, P(_abi.State)], C.c_int),
            "jbgpu_world_set_state": ([C.c_void_p, P(_abi.State)], C.c_int),
            "jbgpu_world_get_pairs": ([C.c_void_p, _abi.u64p, C.c_int32, _abi.i32p], C.c_int),
            "jbgpu_world_get_manifolds": ([C.c_void_p, P(_abi.Manifolds)], C.c_int),
            "jbgpu_world_set_manifolds": ([C.c_void_p, P(_abi.Manifolds)], C.c_int),
            "jbgpu_world_get_solver_order": ([C.c_void_p, _abi.i32p, C.c_int32, _abi.i32p], C.c_int),
            "jbgpu_world_counters": ([C.c_void_p, P(_abi.Counters)], C.c_int),
            "jbgpu_world_apply_forces": ([C.c_void_p, _abi.f32p, _abi.f32p], C.c_int),
            "jbgpu_world_get_transforms": ([C.c_void_p, _abi.f32p], C.c_int),
            "jbgpu_world_set_profiling": ([C.c_void_p, C.c_int32], C.c_int),
            "jbgpu_world_timer": ([C.c_void_p, C.c_int32, C.POINTER(C.c_double)], C.c_int),
            "jbgpu_world_add_point2point": ([C.c_void_p, C.c_int32, C.c_int32, _abi.f32p, _abi.f32p,
                                             C.POINTER(C.c_int32)], C.c_int),
            "jbgpu_world_set_joint_setting": ([C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_float], C.c_int),
            "jbgpu_world_get_joint_impulses": ([C.c_void_p, _abi.f32p, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
            "jbgpu_world_ray_test": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                      C.c_int32, C.c_void_p], C.c_int),
            "jbgpu_world_set_ray_replay": ([C.c_void_p, C.c_int32], C.c_int),
            "jbgpu_world_convex_sweep_test": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                               C.c_int32, C.c_int32, C.c_int32, C.c_void_p], C.c_int),
            "jbgpu_world_set_graph": ([C.c_void_p, C.c_int32], C.c_int),
            "jbgpu_world_graph_status": ([C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_char_p)], C.c_int),
            "jbgpu_world_add_cone_twist": ([C.c_void_p, C.c_int32, C.c_int32, _abi.f32p, _abi.f32p, C.POINTER(C.c_int32)],
                                           C.c_int),
            "jbgpu_world_set_cone_twist_limit": ([C.c_void_p, C.c_int32] + [C.c_float] * 6, C.c_int),
            "jbgpu_world_set_cone_twist_angular_only": ([C.c_void_p, C.c_int32, C.c_int32], C.c_int),
            "jbgpu_world_add_slider": ([C.c_void_p, C.c_int32, C.c_int32, _abi.f32p, _abi.f32p, C.c_int32,
                                       C.POINTER(C.c_int32)], C.c_int),
            "jbgpu_world_set_slider_params": ([C.c_void_p, C.c_int32, _abi.f32p], C.c_int),
            "jbgpu_world_get_slider_params": ([C.c_void_p, C.c_int32, _abi.f32p], C.c_int),
            "jbgpu_world_add_generic6dof": ([C.c_void_p, C.c_int32, C.c_int32, _abi.f32p, _abi.f32p, C.c_int32,
                                            C.POINTER(C.c_int32)], C.c_int),
            "jbgpu_world_set_6dof_limit": ([C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float], C.c_int),
            "jbgpu_world_set_6dof_linear_motor": ([C.c_void_p, C.c_int32] + [C.c_float] * 3, C.c_int),
            "jbgpu_world_set_6dof_angular_motor": ([C.c_void_p, C.c_int32, C.c_int32, C.c_int32] + [C.c_float] * 7,
                                                   C.c_int),
            "jbgpu_world_add_hinge": ([C.c_void_p, C.c_int32, C.c_int32, _abi.f32p, _abi.f32p, C.POINTER(C.c_int32)],
                                      C.c_int),
            "jbgpu_world_set_hinge_limit": ([C.c_void_p, C.c_int32] + [C.c_float] * 5, C.c_int),
            "jbgpu_world_enable_hinge_motor": ([C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float], C.c_int),
            "jbgpu_world_set_hinge_angular_only": ([C.c_void_p, C.c_int32, C.c_int32], C.c_int),
            "jbgpu_world_phase_times": ([C.c_void_p, P(C.c_double), C.c_int32, _abi.i32p], C.c_int),
            "jbgpu_world_profile_counters": ([C.c_void_p, P(_abi.Counters), C.c_int32, _abi.i32p], C.c_int),
            "jbgpu_world_narrowphase_static": ([C.c_void_p, C.c_int32], C.c_int),
            "jbgpu_mlp_create": ([C.c_int32, C.c_uint64, P(C.c_void_p)], C.c_int),
            "jbgpu_mlp_destroy": ([C.c_void_p], C.c_int),
            "jbgpu_mlp_get_params": ([C.c_void_p, _abi.f32p, _abi.f32p], C.c_int),
            "jbgpu_mlp_set_params": ([C.c_void_p, _abi.f32p, _abi.f32p], C.c_int),
            "jbgpu_mlp_forward": ([C.c_void_p, _abi.f32p, C.c_int32, _abi.f32p], C.c_int),
            "jbgpu_mlp_gradients": ([C.c_void_p, _abi.f32p, _abi.f32p, C.c_int32, _abi.f32p, _abi.f32p], C.c_int),
            "jbgpu_mlp_load_samples": ([C.c_void_p, _abi.f32p, _abi.f32p, C.c_int32], C.c_int),
            "jbgpu_mlp_train": ([C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_uint64, _abi.f32p], C.c_int),
            "jbgpu_world_set_warmstart_mlp": ([C.c_void_p, C.c_void_p], C.c_int),
            "jbgpu_world_set_solver_iterations": ([C.c_void_p, C.c_int32, C.c_float, C.c_int32], C.c_int),
            "jbgpu_world_get_residual_trace": ([C.c_void_p, _abi.f32p, C.c_int32, _abi.i32p], C.c_int),
            "jbgpu_world_set_ccd": ([C.c_void_p, _abi.i32p, _abi.f32p, _abi.f32p, C.c_int32], C.c_int),
            "jbgpu_world_refit_mesh": ([C.c_void_p, C.c_int32, _abi.f32p, C.c_int32], C.c_int),
            "jbgpu_world_set_gravity": ([C.c_void_p, _abi.f32p], C.c_int),
            "jbgpu_world_remove_bodies": ([C.c_void_p, _abi.i32p, C.c_int32], C.c_int),
            "jbgpu_world_apply_impulses": ([C.c_void_p, _abi.i32p, _abi.f32p, _abi.f32p, _abi.f32p, C.c_int32], C.c_int),
            "jbgpu_world_set_body_properties": ([C.c_void_p, _abi.i32p, C.c_int32] + [_abi.f32p] * 6, C.c_int),
            "jbgpu_world_remove_joint": ([C.c_void_p, C.c_int32], C.c_int),
            "jbgpu_world_get_interpolated_transforms": ([C.c_void_p, _abi.f32p], C.c_int),
            "jbgpu_world_set_internal_tick_callback": ([C.c_void_p, _abi.TICK_CALLBACK, C.c_void_p], C.c_int),
            "jbgpu_world_set_body_gravity": ([C.c_void_p, _abi.i32p, _abi.f32p, C.c_int32], C.c_int),
            "jbgpu_world_mesh_bvh": ([C.c_void_p, C.c_int32, _abi.i32p, C.c_int32, _abi.i32p, _abi.f32p], C.c_int),
            "jbgpu_world_set_sample_logging": ([C.c_void_p, C.c_int32], C.c_int),
            "jbgpu_world_get_samples": ([C.c_void_p, _abi.f32p, _abi.f32p, C.c_int32, _abi.i32p], C.c_int),
        }
        for name, (args, res) in sigs.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


EXPORTED = [
    "jbgpu_version", "jbgpu_launch_count", "jbgpu_last_error", "jbgpu_config_default", "jbgpu_shape_local_inertia", "jbgpu_world_create",
    "jbgpu_world_destroy", "jbgpu_world_add_shape", "jbgpu_world_add_shapes", "jbgpu_world_add_bodies",
    "jbgpu_world_num_bodies", "jbgpu_world_step_simulation", "jbgpu_world_step", "jbgpu_world_stage",
    "jbgpu_world_synchronize", "jbgpu_world_get_state", "jbgpu_world_set_state", "jbgpu_world_get_pairs",
    "jbgpu_world_get_manifolds", "jbgpu_world_set_manifolds", "jbgpu_world_get_solver_order", "jbgpu_world_counters",
    "jbgpu_world_apply_forces", "jbgpu_world_get_transforms", "jbgpu_world_set_profiling", "jbgpu_world_phase_times",
    "jbgpu_world_profile_counters", "jbgpu_world_timer", "jbgpu_world_add_point2point", "jbgpu_world_set_joint_setting",
    "jbgpu_world_get_joint_impulses", "jbgpu_world_add_hinge", "jbgpu_world_set_hinge_limit",
    "jbgpu_world_enable_hinge_motor", "jbgpu_world_set_hinge_angular_only", "jbgpu_world_ray_test",
    "jbgpu_world_set_ray_replay", "jbgpu_world_convex_sweep_test", "jbgpu_world_set_graph", "jbgpu_world_graph_status", "jbgpu_world_add_generic6dof",
    "jbgpu_world_set_6dof_limit", "jbgpu_world_set_6dof_linear_motor", "jbgpu_world_set_6dof_angular_motor",
    "jbgpu_world_add_cone_twist", "jbgpu_world_set_cone_twist_limit", "jbgpu_world_set_cone_twist_angular_only",
    "jbgpu_world_add_slider", "jbgpu_world_set_slider_params", "jbgpu_world_get_slider_params",
    "jbgpu_world_get_residual_trace", "jbgpu_world_set_ccd", "jbgpu_shape_mesh_bvh", "jbgpu_world_refit_mesh",
    "jbgpu_world_mesh_bvh", "jbgpu_world_set_gravity", "jbgpu_world_set_body_gravity", "jbgpu_world_remove_bodies",
    "jbgpu_world_apply_impulses", "jbgpu_world_set_body_properties", "jbgpu_world_set_internal_tick_callback",
    "jbgpu_world_remove_joint", "jbgpu_world_get_interpolated_transforms",
]


def launch_count():
    return lib().jbgpu_launch_count()


MLP_INPUTS, MLP_OUTPUTS, MLP_PARAMS, MLP_NORM = 24, 3, 5955, 55


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Mlp:
    """The warm-start MLP (jbgpu_mlp_*): 24 -> 64 -> 64 -> 3 on the device's tensor cores."""

    def __init__(self, device=0, seed=0):
        h = C.c_void_p()
        check(lib().jbgpu_mlp_create(device, seed, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().jbgpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.zeros(MLP_PARAMS, np.float32)
        nrm = np.zeros(MLP_NORM, np.float32)
        check(lib().jbgpu_mlp_get_params(self.h, _abi._ptr(p, _abi.f32p), _abi._ptr(nrm, _abi.f32p)))
        return p, nrm

    def set_params(self, params=None, norm=None):
        p = None if params is None else _f32(params, (MLP_PARAMS,))
        n = None if norm is None else _f32(norm, (MLP_NORM,))
        check(lib().jbgpu_mlp_set_params(self.h, _abi._ptr(p, _abi.f32p), _abi._ptr(n, _abi.f32p)))

    def forward(self, x):
        x = _f32(x)
        y = np.zeros((len(x), MLP_OUTPUTS), np.float32)
        check(lib().jbgpu_mlp_forward(self.h, _abi._ptr(x, _abi.f32p), len(x), _abi._ptr(y, _abi.f32p)))
        return y

    def gradients(self, x, t):
        x, t = _f32(x), _f32(t)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        check(lib().jbgpu_mlp_gradients(self.h, _abi._ptr(x, _abi.f32p), _abi._ptr(t, _abi.f32p), len(x),
                                        _abi._ptr(g, _abi.f32p), _abi._ptr(loss, _abi.f32p)))
        return g, float(loss[0])

    def train(self, x, t, epochs, batch=1024, lr=1e-3, seed=0):
        x, t = _f32(x), _f32(t)
        check(lib().jbgpu_mlp_load_samples(self.h, _abi._ptr(x, _abi.f32p), _abi._ptr(t, _abi.f32p), len(x)))
        losses = np.zeros(epochs, np.float32)
        check(lib().jbgpu_mlp_train(self.h, epochs, batch, lr, seed, _abi._ptr(losses, _abi.f32p)))
        return losses

PHASES = ["predict", "aabb", "pair_count", "pair_fill", "narrow_gjk", "narrow_epa", "islands", "colour", "setup", "pgs",
          "integrate", "activation", "gravity", "concave"]


def check(rc):
    if rc != 0:
        msg = lib().jbgpu_last_error()
        raise JbgpuError(rc, msg.decode() if msg else "")
    return rc


class GpuWorld:
    _tick = None

    def __init__(self, scene=None, config=None):
        cfg = config if config is not None else _abi.default_config(**(scene.config if scene else {}))
        self._cfg = cfg
        h = C.c_void_p()
        check(lib().jbgpu_world_create(C.byref(cfg), C.byref(h)))
        self.h = h
        if scene is not None:
            self.add_scene(scene)
            self.add_scene_joints(scene)
            ccd = scene.meta.get("ccd")
            if ccd:
                self.set_ccd(ccd["bodies"], ccd["threshold"], ccd["radius"])

    def close(self):
        if getattr(self, "h", None):
            lib().jbgpu_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene):
        descs = scene.shape_descs()
        check(lib().jbgpu_world_add_shapes(self.h, descs, len(descs), None))
        b, ptr = scene.body_descs_ptr()
        check(lib().jbgpu_world_add_bodies(self.h, ptr, len(b), None))

    def add_point2point(self, a, b, pivot_a, pivot_b):
        """Point-to-point joint between bodies a and b (b = -1: the fixed body); returns its id."""
        pa = np.ascontiguousarray(pivot_a, np.float32)
        pb = np.ascontiguousarray(pivot_b, np.float32)
        jid = C.c_int32()
        check(lib().jbgpu_world_add_point2point(self.h, a, b, pa.ctypes.data_as(_abi.f32p), pb.ctypes.data_as(_abi.f32p),
                                                C.byref(jid)))
        return jid.value

    def set_joint_setting(self, jid, tau=0.3, damping=1.0, impulse_clamp=0.0):
        check(lib().jbgpu_world_set_joint_setting(self.h, jid, tau, damping, impulse_clamp))

    def get_interpolated_transforms(self):
        """synchronizeMotionStates' transforms (jbgpu_world_get_interpolated_transforms), (n, 12)."""
        out = np.zeros((max(self.n_bodies, 1), 12), np.float32)
        check(lib().jbgpu_world_get_interpolated_transforms(self.h, out.ctypes.data_as(_abi.f32p)))
        return out[:self.n_bodies]

    def remove_joint(self, jid):
        """DiscreteDynamicsWorld.removeConstraint: the joints after it move down one id."""
        check(lib().jbgpu_world_remove_joint(self.h, jid))

    def joint_impulses(self):
        n = C.c_int32()
        check(lib().jbgpu_world_get_joint_impulses(self.h, None, 0, C.byref(n)))
        out = np.zeros(max(n.value, 1), np.float32)
        check(lib().jbgpu_world_get_joint_impulses(self.h, out.ctypes.data_as(_abi.f32p), n.value, C.byref(n)))
        return out[:n.value].copy()

    def add_hinge(self, a, b, frame_a, frame_b):
        """Hinge between bodies a and b (b = -1: the fixed body) with the constraint frames as
        HingeConstraint holds them (12 floats each: basis row-major, origin); returns its id."""
        fa = np.ascontiguousarray(frame_a, np.float32).reshape(12)
        fb = np.ascontiguousarray(frame_b, np.float32).reshape(12)
        jid = C.c_int32()
        check(lib().jbgpu_world_add_hinge(self.h, a, b, fa.ctypes.data_as(_abi.f32p), fb.ctypes.data_as(_abi.f32p),
                                          C.byref(jid)))
        return jid.value

    def set_hinge_limit(self, jid, low, high, softness=0.9, bias_factor=0.3, relaxation_factor=1.0):
        check(lib().jbgpu_world_set_hinge_limit(self.h, jid, low, high, softness, bias_factor, relaxation_factor))

    def enable_hinge_motor(self, jid, enable, target_velocity, max_motor_impulse):
        check(lib().jbgpu_world_enable_hinge_motor(self.h, jid, 1 if enable else 0, target_velocity, max_motor_impulse))

    def set_hinge_angular_only(self, jid, on):
        check(lib().jbgpu_world_set_hinge_angular_only(self.h, jid, 1 if on else 0))

    def ray_test(self, ray_from, ray_to, world=None, group=1, mask=-1):
        """CollisionWorld.rayTest with a ClosestRayResultCallback per ray: ray_from / ray_to (n, 3),
        world (n,) batch world per ray or None.  Returns a RAY_HIT_DTYPE array (body -1: no hit)."""
        f = np.ascontiguousarray(ray_from, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(ray_to, np.float32).reshape(-1, 3)
        n = len(f)
        if len(t) != n:
            raise ValueError("ray_from and ray_to differ in length")
        out = np.zeros(n, _abi.RAY_HIT_DTYPE)
        wp = None
        if world is not None:
            wa = np.ascontiguousarray(world, np.int32).reshape(n)
            wp = wa.ctypes.data
        check(lib().jbgpu_world_ray_test(self.h, f.ctypes.data, t.ctypes.data, wp, n, group, mask, 0, out.ctypes.data))
        return out

    def ray_test_device(self, from_ptr, to_ptr, n, hits_ptr, world_ptr=None, group=1, mask=-1):
        """rayTest on device buffers (raw pointers); queued on the world's stream."""
        check(lib().jbgpu_world_ray_test(self.h, from_ptr, to_ptr, world_ptr, n, group, mask, 1, hits_ptr))

    def convex_sweep_test(self, shape, xf_from, xf_to, world=None, group=1, mask=-1):
        """CollisionWorld.convexSweepTest with a ClosestConvexResultCallback per sweep of the convex
        shape id `shape`: xf_from / xf_to (n, 12) transforms (basis row-major, origin), world (n,)
        batch world per sweep or None.  Returns a RAY_HIT_DTYPE array (body -1: no hit; -2: the
        sweep reached a static plane, where the reference throws)."""
        f = np.ascontiguousarray(xf_from, np.float32).reshape(-1, 12)
        t = np.ascontiguousarray(xf_to, np.float32).reshape(-1, 12)
        n = len(f)
        if len(t) != n:
            raise ValueError("xf_from and xf_to differ in length")
        out = np.zeros(n, _abi.RAY_HIT_DTYPE)
        wp = None
        if world is not None:
            wa = np.ascontiguousarray(world, np.int32).reshape(n)
            wp = wa.ctypes.data
        check(lib().jbgpu_world_convex_sweep_test(self.h, shape, f.ctypes.data, t.ctypes.data, wp, n, group, mask, 0,
                                                  out.ctypes.data))
        return out

    def convex_sweep_test_device(self, shape, from_ptr, to_ptr, n, hits_ptr, world_ptr=None, group=1, mask=-1):
        """convexSweepTest on device buffers (raw pointers); queued on the world's stream."""
        check(lib().jbgpu_world_convex_sweep_test(self.h, shape, from_ptr, to_ptr, world_ptr, n, group, mask, 1, hits_ptr))

    def set_graph(self, on):
        """Replay the step as CUDA graphs (bit-identical to launching its kernels)."""
        check(lib().jbgpu_world_set_graph(self.h, 1 if on else 0))

    def graph_status(self):
        n = C.c_int32()
        e = C.c_char_p()
        check(lib().jbgpu_world_graph_status(self.h, C.byref(n), C.byref(e)))
        return n.value, (e.value or b"").decode()

    def set_ray_replay(self, all_rays):
        check(lib().jbgpu_world_set_ray_replay(self.h, 1 if all_rays else 0))

    def add_slider(self, a, b, frame_a, frame_b, use_linear_reference_frame_a=True):
        """Slider joint with frames as 12 floats each (basis row-major, origin); returns its id."""
        fa = np.ascontiguousarray(frame_a, np.float32).reshape(12)
        fb = np.ascontiguousarray(frame_b, np.float32).reshape(12)
        jid = C.c_int32()
        check(lib().jbgpu_world_add_slider(self.h, a, b, fa.ctypes.data_as(_abi.f32p), fb.ctypes.data_as(_abi.f32p),
                                           1 if use_linear_reference_frame_a else 0, C.byref(jid)))
        return jid.value

    def slider_params(self, jid):
        p = np.zeros(28, np.float32)
        check(lib().jbgpu_world_get_slider_params(self.h, jid, p.ctypes.data_as(_abi.f32p)))
        return p

    def set_slider_params(self, jid, params):
        p = np.ascontiguousarray(params, np.float32).reshape(28)
        check(lib().jbgpu_world_set_slider_params(self.h, jid, p.ctypes.data_as(_abi.f32p)))

    def add_cone_twist(self, a, b, frame_a, frame_b):
        """Cone-twist joint with frames as 12 floats each (basis row-major, origin); returns its id."""
        fa = np.ascontiguousarray(frame_a, np.float32).reshape(12)
        fb = np.ascontiguousarray(frame_b, np.float32).reshape(12)
        jid = C.c_int32()
        check(lib().jbgpu_world_add_cone_twist(self.h, a, b, fa.ctypes.data_as(_abi.f32p), fb.ctypes.data_as(_abi.f32p),
                                               C.byref(jid)))
        return jid.value

    def set_cone_limit(self, jid, swing1, swing2, twist, softness=0.8, bias_factor=0.3, relaxation_factor=1.0):
        check(lib().jbgpu_world_set_cone_twist_limit(self.h, jid, swing1, swing2, twist, softness, bias_factor,
                                                     relaxation_factor))

    def set_cone_angular_only(self, jid, on):
        check(lib().jbgpu_world_set_cone_twist_angular_only(self.h, jid, 1 if on else 0))

    def add_generic6dof(self, a, b, frame_a, frame_b, use_linear_reference_frame_a=True):
        """Generic 6-dof joint with frames as 12 floats each (basis row-major, origin); returns its id."""
        fa = np.ascontiguousarray(frame_a, np.float32).reshape(12)
        fb = np.ascontiguousarray(frame_b, np.float32).reshape(12)
        jid = C.c_int32()
        check(lib().jbgpu_world_add_generic6dof(self.h, a, b, fa.ctypes.data_as(_abi.f32p), fb.ctypes.data_as(_abi.f32p),
                                                1 if use_linear_reference_frame_a else 0, C.byref(jid)))
        return jid.value

    def set_6dof_limit(self, jid, axis, lo, hi):
        check(lib().jbgpu_world_set_6dof_limit(self.h, jid, axis, lo, hi))

    def set_6dof_linear_motor(self, jid, softness, damping, restitution):
        check(lib().jbgpu_world_set_6dof_linear_motor(self.h, jid, softness, damping, restitution))

    def set_6dof_angular_motor(self, jid, axis, enable, target_velocity, max_motor_force, max_limit_force=300.0,
                               damping=1.0, softness=0.5, erp=0.5, bounce=0.0):
        check(lib().jbgpu_world_set_6dof_angular_motor(self.h, jid, axis, 1 if enable else 0, target_velocity,
                                                       max_motor_force, max_limit_force, damping, softness, erp, bounce))

    def add_scene_joints(self, scene):
        for j in scene.meta.get("joints", []):
            if j.get("type") == "slider":
                jid = self.add_slider(j["a"], j["b"], j["frame_a"], j["frame_b"], j.get("use_a", True))
                if "params" in j:
                    self.set_slider_params(jid, j["params"])
                continue
            if j.get("type") == "cone":
                jid = self.add_cone_twist(j["a"], j["b"], j["frame_a"], j["frame_b"])
                if "limit" in j:
                    self.set_cone_limit(jid, *j["limit"])
                if j.get("angular_only"):
                    self.set_cone_angular_only(jid, True)
                continue
            if j.get("type") == "6dof":
                jid = self.add_generic6dof(j["a"], j["b"], j["frame_a"], j["frame_b"], j.get("use_a", True))
                for axis, lo, hi in j.get("limits", []):
                    self.set_6dof_limit(jid, axis, lo, hi)
                if "linear_motor" in j:
                    self.set_6dof_linear_motor(jid, *j["linear_motor"])
                for m in j.get("angular_motors", []):
                    self.set_6dof_angular_motor(jid, *m)
                continue
            if j.get("type") == "hinge":
                jid = self.add_hinge(j["a"], j["b"], j["frame_a"], j["frame_b"])
                if "limit" in j:
                    self.set_hinge_limit(jid, *j["limit"])
                if "motor" in j:
                    self.enable_hinge_motor(jid, *j["motor"])
                if j.get("angular_only"):
                    self.set_hinge_angular_only(jid, True)
                continue
            jid = self.add_point2point(j["a"], j["b"], j["pivot_a"], j["pivot_b"])
            if "setting" in j:
                self.set_joint_setting(jid, *j["setting"])

    @property
    def n_bodies(self):
        n = C.c_int32()
        check(lib().jbgpu_world_num_bodies(self.h, C.byref(n)))
        return n.value

    def step(self, dt, substeps=1):
        rc = lib().jbgpu_world_step(self.h, dt, substeps)
        if self._tick:
            self._tick.reraise()
        check(rc)

    def step_simulation(self, time_step, max_sub_steps=1, fixed_time_step=1.0 / 60.0):
        n = C.c_int32()
        rc = lib().jbgpu_world_step_simulation(self.h, time_step, max_sub_steps, fixed_time_step, C.byref(n))
        if self._tick:
            self._tick.reraise()
        check(rc)
        return n.value

    def set_internal_tick_callback(self, cb):
        """DynamicsWorld.setInternalTickCallback: cb(world, time_step) after every substep; None removes it."""
        t = None if cb is None else _abi.TickTrampoline(self, cb)
        check(lib().jbgpu_world_set_internal_tick_callback(self.h, _abi.TICK_CALLBACK() if t is None else t.fn, None))
        self._tick = t

    def set_body_properties(self, bodies, **props):
        """RigidBody.setDamping / setSleepingThresholds, CollisionObject.setFriction / setRestitution
        after the bodies were added (jbgpu_world_set_body_properties); keywords are
        _abi.BODY_PROPERTIES, each a scalar or one value per body."""
        b, arrs = _abi.body_property_arrays(bodies, props)
        ptr = [None if a is None else a.ctypes.data_as(_abi.f32p) for a in arrs]
        check(lib().jbgpu_world_set_body_properties(self.h, b.ctypes.data_as(_abi.i32p), len(b), *ptr))

    def stage(self, stage, dt=1.0 / 60.0):
        check(lib().jbgpu_world_stage(self.h, stage, dt))

    def synchronize(self):
        check(lib().jbgpu_world_synchronize(self.h))

    def get_state(self):
        sb = _abi.StateBuffers(self.n_bodies)
        check(lib().jbgpu_world_get_state(self.h, C.byref(sb.struct)))
        return sb.copy_arrays()

    def set_state(self, arrays):
        arrays = {k: v for k, v in arrays.items() if k != "island_tag"}
        sb = _abi.StateBuffers.from_arrays(arrays)
        check(lib().jbgpu_world_set_state(self.h, C.byref(sb.struct)))

    def get_pairs(self):
        n = C.c_int32()
        lib().jbgpu_world_get_pairs(self.h, None, 0, C.byref(n))
        keys = np.zeros(max(1, n.value), np.uint64)
        check(lib().jbgpu_world_get_pairs(self.h, keys.ctypes.data_as(_abi.u64p), len(keys), C.byref(n)))
        return keys[:n.value]

    def get_manifolds(self):
        n = C.c_int32()
        lib().jbgpu_world_get_pairs(self.h, None, 0, C.byref(n))
        mb = _abi.ManifoldBuffers(max(1, n.value))
        check(lib().jbgpu_world_get_manifolds(self.h, C.byref(mb.struct)))
        return mb.view()

    def set_manifolds(self, m):
        mb = _abi.ManifoldBuffers.from_arrays(m["keys"], m["flags"], m["num_points"], m["points"])
        check(lib().jbgpu_world_set_manifolds(self.h, C.byref(mb.struct)))

    def solver_order(self):
        n = C.c_int32()
        lib().jbgpu_world_get_solver_order(self.h, None, 0, C.byref(n))
        out = np.zeros(max(1, n.value), np.int32)
        check(lib().jbgpu_world_get_solver_order(self.h, out.ctypes.data_as(_abi.i32p), len(out), C.byref(n)))
        return out[:n.value]

    def set_solver_iterations(self, num_iterations, residual=0.0, max_iterations=0):
        check(lib().jbgpu_world_set_solver_iterations(self.h, num_iterations, residual, max_iterations))

    def apply_impulses(self, bodies, impulses=None, rel_pos=None, torque_impulses=None):
        """RigidBody.applyCentralImpulse / applyImpulse (rel_pos given) / applyTorqueImpulse for
        distinct bodies (jbgpu_world_apply_impulses)."""
        b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
        arrs = [None if a is None else np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float32).reshape(-1, 3),
                                                                            (len(b), 3)), np.float32)
                for a in (impulses, rel_pos, torque_impulses)]
        ptr = [None if a is None else a.ctypes.data_as(_abi.f32p) for a in arrs]
        check(lib().jbgpu_world_apply_impulses(self.h, b.ctypes.data_as(_abi.i32p), ptr[0], ptr[1], ptr[2], len(b)))

    def remove_bodies(self, bodies):
        """DiscreteDynamicsWorld.removeRigidBody for the given bodies (jbgpu_world_remove_bodies):
        the bodies after each removed one move down."""
        b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
        check(lib().jbgpu_world_remove_bodies(self.h, b.ctypes.data_as(_abi.i32p), len(b)))

    def set_gravity(self, g):
        """DiscreteDynamicsWorld.setGravity (jbgpu_world_set_gravity)."""
        a = np.ascontiguousarray(g, np.float32).reshape(3)
        check(lib().jbgpu_world_set_gravity(self.h, a.ctypes.data_as(_abi.f32p)))

    def set_body_gravity(self, bodies, acceleration):
        """RigidBody.setGravity for the given bodies (one acceleration each, or one for all)."""
        b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(acceleration, np.float32).reshape(-1, 3), (len(b), 3)),
                                 np.float32)
        check(lib().jbgpu_world_set_body_gravity(self.h, b.ctypes.data_as(_abi.i32p), a.ctypes.data_as(_abi.f32p), len(b)))

    def refit_mesh(self, shape, points):
        """New positions of a triangle mesh's vertices: BvhTriangleMeshShape.refitTree and
        updateSingleAabb of its bodies (jbgpu_world_refit_mesh)."""
        p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        check(lib().jbgpu_world_refit_mesh(self.h, int(shape), p.ctypes.data_as(_abi.f32p), len(p)))

    def mesh_bvh(self, shape):
        """The world's current tree of a triangle-mesh shape: (nodes (n, 4) int32, local aabb (6,))."""
        n = C.c_int32()
        aabb = np.zeros(6, np.float32)
        rc = lib().jbgpu_world_mesh_bvh(self.h, int(shape), None, 0, C.byref(n), aabb.ctypes.data_as(_abi.f32p))
        if rc not in (0, _abi.ERR_CAPACITY):
            check(rc)
        nodes = np.zeros((n.value, 4), np.int32)
        check(lib().jbgpu_world_mesh_bvh(self.h, int(shape), nodes.ctypes.data_as(_abi.i32p), n.value, C.byref(n),
                                         aabb.ctypes.data_as(_abi.f32p)))
        return nodes, aabb

    def set_ccd(self, bodies, motion_threshold, swept_sphere_radius):
        """CollisionObject.setCcdMotionThreshold / setCcdSweptSphereRadius for the given bodies."""
        b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
        t = np.ascontiguousarray(np.broadcast_to(np.float32(motion_threshold) if np.isscalar(motion_threshold)
                                                 else motion_threshold, b.shape), np.float32)
        r = np.ascontiguousarray(np.broadcast_to(np.float32(swept_sphere_radius) if np.isscalar(swept_sphere_radius)
                                                 else swept_sphere_radius, b.shape), np.float32)
        check(lib().jbgpu_world_set_ccd(self.h, b.ctypes.data_as(_abi.i32p), t.ctypes.data_as(_abi.f32p),
                                        r.ctypes.data_as(_abi.f32p), len(b)))

    def residual_trace(self):
        """(max |delta lambda|, max |lambda|) per iteration of the last step's residual-mode solve."""
        n = C.c_int32()
        check(lib().jbgpu_world_get_residual_trace(self.h, None, 0, C.byref(n)))
        out = np.zeros((max(1, n.value), 2), np.float32)
        check(lib().jbgpu_world_get_residual_trace(self.h, out.ctypes.data_as(_abi.f32p), len(out), C.byref(n)))
        return out[:n.value]

    def set_warmstart_mlp(self, mlp):
        self._mlp = mlp
        check(lib().jbgpu_world_set_warmstart_mlp(self.h, mlp.h if mlp is not None else None))

    def set_sample_logging(self, on=True, all_points=False):
        """Training samples of every solve: converged islands' points (all_points False) or every
        point's impulses after the last iteration run (all_points True)."""
        check(lib().jbgpu_world_set_sample_logging(self.h, (2 if all_points else 1) if on else 0))

    def get_samples(self):
        n = C.c_int32()
        check(lib().jbgpu_world_get_samples(self.h, None, None, 0, C.byref(n)))
        x = np.zeros((max(1, n.value), MLP_INPUTS), np.float32)
        t = np.zeros((max(1, n.value), MLP_OUTPUTS), np.float32)
        check(lib().jbgpu_world_get_samples(self.h, _abi._ptr(x, _abi.f32p), _abi._ptr(t, _abi.f32p), len(x),
                                            C.byref(n)))
        return x[:n.value], t[:n.value]

    def counters(self):
        c = _abi.Counters()
        check(lib().jbgpu_world_counters(self.h, C.byref(c)))
        return c.as_dict()

    def apply_forces(self, force=None, torque=None):
        f = None if force is None else np.ascontiguousarray(force, np.float32)
        t = None if torque is None else np.ascontiguousarray(torque, np.float32)
        check(lib().jbgpu_world_apply_forces(self.h, None if f is None else f.ctypes.data_as(_abi.f32p),
                                             None if t is None else t.ctypes.data_as(_abi.f32p)))

    def get_transforms(self, out=None):
        if out is None:
            out = np.zeros((self.n_bodies, 12), np.float32)
        check(lib().jbgpu_world_get_transforms(self.h, out.ctypes.data_as(_abi.f32p)))
        return out

    def set_profiling(self, max_steps):
        check(lib().jbgpu_world_set_profiling(self.h, max_steps))

    def timer_start(self):
        """Records the device timer's start event on the world's stream."""
        check(lib().jbgpu_world_timer(self.h, 0, None))

    def timer_stop(self):
        """Device milliseconds since timer_start (records the end event and waits for it)."""
        ms = C.c_double(0.0)
        check(lib().jbgpu_world_timer(self.h, 1, C.byref(ms)))
        return ms.value

    def phase_times(self):
        """({phase: total device ms}, profiled steps, whole-window device ms)."""
        ms = (C.c_double * (len(PHASES) + 1))()
        n = C.c_int32()
        check(lib().jbgpu_world_phase_times(self.h, ms, len(PHASES) + 1, C.byref(n)))
        return dict(zip(PHASES, list(ms)[:len(PHASES)])), n.value, ms[len(PHASES)]

    def profile_counters(self):
        n = C.c_int32()
        check(lib().jbgpu_world_profile_counters(self.h, None, 0, C.byref(n)))
        arr = (_abi.Counters * max(1, n.value))()
        check(lib().jbgpu_world_profile_counters(self.h, arr, len(arr), C.byref(n)))
        return [arr[i].as_dict() for i in range(n.value)]


def shape_local_inertia(shape_dict, mass):
    from .scenes import Scene
    sc = Scene("one", 0, 0, {}, [shape_dict], np.zeros(0))
    d = sc.shape_descs()
    out = np.zeros(3, np.float32)
    check(lib().jbgpu_shape_local_inertia(C.byref(d[0]), mass, out.ctypes.data_as(_abi.f32p)))
    return out


def mesh_bvh(mesh_dict):
    """The quantized tree the library builds for a triangle-mesh shape dict: (nodes (n, 4) int32 in
    walk order, local aabb (6,) float32) - see jbgpu_shape_mesh_bvh."""
    from .scenes import shape_desc_array
    d = shape_desc_array([mesh_dict])
    n = C.c_int32()
    aabb = np.zeros(6, np.float32)
    rc = lib().jbgpu_shape_mesh_bvh(C.byref(d[0]), None, 0, C.byref(n), aabb.ctypes.data_as(_abi.f32p))
    if rc not in (_abi.OK, _abi.ERR_CAPACITY):
        check(rc)
    nodes = np.zeros((max(n.value, 1), 4), np.int32)
    check(lib().jbgpu_shape_mesh_bvh(C.byref(d[0]), nodes.ctypes.data_as(_abi.i32p), len(nodes), C.byref(n),
                                     aabb.ctypes.data_as(_abi.f32p)))
    return nodes[:n.value], aabb
