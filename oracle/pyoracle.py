"""ORACLE (test infrastructure only): ctypes wrapper over oracle/_build/liboracle.so, the
single-threaded CPU restatement of the reference's step.  Imported by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg; never by the product."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REPO = os.path.dirname(_HERE)
sys.path.insert(0, os.path.join(_REPO, "libgdx-jbullet_gb300"))
from jbgpu import _abi  # noqa: E402

LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
ORDER_REFERENCE, ORDER_COLOUR, ORDER_EXPLICIT = 0, 1, 2
_lib = None


def build():
    subprocess.check_call(["make", "-s", "-j8"], cwd=_HERE)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(_abi.Config)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_add_shape.argtypes = [C.c_void_p, C.POINTER(_abi.ShapeDesc)]
        L.orc_add_bodies.argtypes = [C.c_void_p, C.POINTER(_abi.BodyDesc), C.c_int]
        L.orc_step_simulation.argtypes = [C.c_void_p, C.c_float, C.c_int, C.c_float]
        L.orc_step.argtypes = [C.c_void_p, C.c_float, C.c_int]
        L.orc_stage.argtypes = [C.c_void_p, C.c_int, C.c_float]
        L.orc_set_order_mode.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_explicit_order.argtypes = [C.c_void_p, _abi.i32p, C.c_int]
        L.orc_set_brute_force.argtypes = [C.c_void_p, C.c_int]
        L.orc_num_bodies.argtypes = [C.c_void_p]
        L.orc_get_state.argtypes = [C.c_void_p, C.POINTER(_abi.State)]
        L.orc_set_state.argtypes = [C.c_void_p, C.POINTER(_abi.State)]
        L.orc_get_manifolds.argtypes = [C.c_void_p, C.POINTER(_abi.Manifolds)]
        L.orc_set_manifolds.argtypes = [C.c_void_p, C.POINTER(_abi.Manifolds)]
        L.orc_get_solver_order.argtypes = [C.c_void_p, _abi.i32p, C.c_int]
        L.orc_counters.argtypes = [C.c_void_p, C.POINTER(_abi.Counters)]
        L.orc_phase_seconds.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.orc_shape_local_inertia.argtypes = [C.POINTER(_abi.ShapeDesc), C.c_float, _abi.f32p]
        L.orc_mesh_bvh.argtypes = [C.POINTER(_abi.ShapeDesc), _abi.i32p, C.c_int, _abi.f32p]
        L.orc_mesh_query.argtypes = [C.POINTER(_abi.ShapeDesc), _abi.f32p, _abi.f32p, _abi.i32p, C.c_int]
        L.orc_gjk.argtypes = [C.POINTER(_abi.ShapeDesc), _abi.f32p, C.POINTER(_abi.ShapeDesc), _abi.f32p, C.c_float, _abi.f32p]
        L.orc_integrate_transform.argtypes = [_abi.f32p, _abi.f32p, _abi.f32p, C.c_float, _abi.f32p]
        L.orc_add_point2point.argtypes = [C.c_void_p, C.c_int, C.c_int, _abi.f32p, _abi.f32p]
        L.orc_set_joint_setting.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float]
        L.orc_get_joint_impulses.argtypes = [C.c_void_p, _abi.f32p, C.c_int]
        L.orc_ray_test.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.orc_add_generic6dof.argtypes = [C.c_void_p, C.c_int, C.c_int, _abi.f32p, _abi.f32p, C.c_int]
        L.orc_set_6dof_limit.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float]
        L.orc_set_6dof_linear_motor.argtypes = [C.c_void_p, C.c_int] + [C.c_float] * 3
        L.orc_set_6dof_angular_motor.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int] + [C.c_float] * 7
        L.orc_add_cone_twist.argtypes = [C.c_void_p, C.c_int, C.c_int, _abi.f32p, _abi.f32p]
        L.orc_set_cone_limit.argtypes = [C.c_void_p, C.c_int] + [C.c_float] * 6
        L.orc_convex_sweep.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                       C.c_void_p]
        L.orc_add_slider.argtypes = [C.c_void_p, C.c_int, C.c_int, _abi.f32p, _abi.f32p, C.c_int]
        L.orc_set_slider_params.argtypes = [C.c_void_p, C.c_int, _abi.f32p]
        L.orc_add_hinge.argtypes = [C.c_void_p, C.c_int, C.c_int, _abi.f32p, _abi.f32p]
        L.orc_set_hinge_limit.argtypes = [C.c_void_p, C.c_int] + [C.c_float] * 5
        L.orc_enable_hinge_motor.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float]
        L.orc_set_hinge_angular_only.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_set_ccd.argtypes = [C.c_void_p, _abi.i32p, _abi.f32p, _abi.f32p, C.c_int]
        L.orc_refit_mesh.argtypes = [C.c_void_p, C.c_int, _abi.f32p, C.c_int]
        L.orc_set_gravity.argtypes = [C.c_void_p, _abi.f32p]
        L.orc_remove_bodies.argtypes = [C.c_void_p, _abi.i32p, C.c_int]
        L.orc_apply_impulses.argtypes = [C.c_void_p, _abi.i32p, _abi.f32p, _abi.f32p, _abi.f32p, C.c_int]
        L.orc_set_body_properties.argtypes = [C.c_void_p, _abi.i32p, C.c_int] + [_abi.f32p] * 6
        L.orc_set_tick_callback.argtypes = [C.c_void_p, _abi.TICK_CALLBACK, C.c_void_p]
        L.orc_set_tick_callback.restype = None
        L.orc_remove_joint.argtypes = [C.c_void_p, C.c_int]
        L.orc_get_interpolated_transforms.argtypes = [C.c_void_p, _abi.f32p]
        L.orc_get_interpolated_transforms.restype = None
        L.orc_set_body_gravity.argtypes = [C.c_void_p, _abi.i32p, _abi.f32p, C.c_int]
        L.orc_world_mesh_bvh.argtypes = [C.c_void_p, C.c_int, _abi.i32p, C.c_int, _abi.f32p]
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(_abi.f32p)


class OracleWorld:
    _tick = None

    def __init__(self, scene=None, config=None, order_mode=ORDER_COLOUR):
        cfg = config if config is not None else _abi.default_config(**(scene.config if scene else {}))
        self._cfg = cfg
        self.h = lib().orc_create(C.byref(cfg))
        self.set_order_mode(order_mode)
        if scene is not None:
            self.add_scene(scene)
            self.add_scene_joints(scene)
            ccd = scene.meta.get("ccd")
            if ccd:
                self.set_ccd(ccd["bodies"], ccd["threshold"], ccd["radius"])

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def add_scene(self, scene):
        descs = scene.shape_descs()
        for i in range(len(descs)):
            lib().orc_add_shape(self.h, C.byref(descs[i]))
        b, ptr = scene.body_descs_ptr()
        lib().orc_add_bodies(self.h, ptr, len(b))

    def add_point2point(self, a, b, pivot_a, pivot_b):
        """Point2PointConstraint between bodies a and b (b = -1: the fixed body); returns its id."""
        pa = np.ascontiguousarray(pivot_a, np.float32)
        pb = np.ascontiguousarray(pivot_b, np.float32)
        return lib().orc_add_point2point(self.h, a, b, _fp(pa), _fp(pb))

    def set_joint_setting(self, jid, tau=0.3, damping=1.0, impulse_clamp=0.0):
        lib().orc_set_joint_setting(self.h, jid, tau, damping, impulse_clamp)

    def get_interpolated_transforms(self):
        """synchronizeMotionStates' transforms, (n, 12)."""
        n = len(self.get_state()["transform"])
        out = np.zeros((max(n, 1), 12), np.float32)
        lib().orc_get_interpolated_transforms(self.h, _fp(out))
        return out[:n]

    def remove_joint(self, jid):
        """DiscreteDynamicsWorld.removeConstraint: the joints after it move down one id."""
        if lib().orc_remove_joint(self.h, jid) != 0:
            raise ValueError("remove_joint: bad joint id")

    def joint_impulses(self):
        n = lib().orc_get_joint_impulses(self.h, None, 0)
        out = np.zeros(max(n, 1), np.float32)
        lib().orc_get_joint_impulses(self.h, _fp(out), n)
        return out[:n].copy()

    def ray_test(self, ray_from, ray_to, world=None, group=1, mask=-1):
        """CollisionWorld.rayTest with a ClosestRayResultCallback per ray (RAY_HIT_DTYPE records)."""
        f = np.ascontiguousarray(ray_from, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(ray_to, np.float32).reshape(-1, 3)
        out = np.zeros(len(f), _abi.RAY_HIT_DTYPE)
        wa = None if world is None else np.ascontiguousarray(world, np.int32).reshape(len(f))
        lib().orc_ray_test(self.h, f.ctypes.data, t.ctypes.data, None if wa is None else wa.ctypes.data, len(f), group,
                           mask, out.ctypes.data)
        return out

    def add_hinge(self, a, b, frame_a, frame_b):
        """HingeConstraint between bodies a and b (b = -1: the fixed body) with the constraint
        frames as the reference holds them (12 floats each: basis row-major, origin)."""
        fa = np.ascontiguousarray(frame_a, np.float32).reshape(12)
        fb = np.ascontiguousarray(frame_b, np.float32).reshape(12)
        return lib().orc_add_hinge(self.h, a, b, _fp(fa), _fp(fb))

    def set_hinge_limit(self, jid, low, high, softness=0.9, bias_factor=0.3, relaxation_factor=1.0):
        lib().orc_set_hinge_limit(self.h, jid, low, high, softness, bias_factor, relaxation_factor)

    def enable_hinge_motor(self, jid, enable, target_velocity, max_motor_impulse):
        lib().orc_enable_hinge_motor(self.h, jid, 1 if enable else 0, target_velocity, max_motor_impulse)

    def set_hinge_angular_only(self, jid, on):
        lib().orc_set_hinge_angular_only(self.h, jid, 1 if on else 0)

    def convex_sweep(self, shape, xf_from, xf_to, world=None, group=1, mask=-1):
        """convexSweepTest with a ClosestConvexResultCallback per sweep of shape `shape` from / to
        transforms (n, 12).  Records as RAY_HIT_DTYPE; body -2 marks a sweep that reached a static
        plane (where the reference throws).  Returns (records, number of such sweeps)."""
        f = np.ascontiguousarray(xf_from, np.float32).reshape(-1, 12)
        t = np.ascontiguousarray(xf_to, np.float32).reshape(-1, 12)
        out = np.zeros(len(f), _abi.RAY_HIT_DTYPE)
        wa = None if world is None else np.ascontiguousarray(world, np.int32).reshape(len(f))
        planes = lib().orc_convex_sweep(self.h, shape, f.ctypes.data, t.ctypes.data, None if wa is None else wa.ctypes.data,
                                        len(f), group, mask, out.ctypes.data)
        return out, planes

    def add_generic6dof(self, a, b, frame_a, frame_b, use_linear_reference_frame_a=True):
        fa = np.ascontiguousarray(frame_a, np.float32).reshape(12)
        fb = np.ascontiguousarray(frame_b, np.float32).reshape(12)
        return lib().orc_add_generic6dof(self.h, a, b, _fp(fa), _fp(fb), 1 if use_linear_reference_frame_a else 0)

    def set_6dof_limit(self, jid, axis, lo, hi):
        lib().orc_set_6dof_limit(self.h, jid, axis, lo, hi)

    def set_6dof_linear_motor(self, jid, softness, damping, restitution):
        lib().orc_set_6dof_linear_motor(self.h, jid, softness, damping, restitution)

    def set_6dof_angular_motor(self, jid, axis, enable, target_velocity, max_motor_force, max_limit_force=300.0,
                               damping=1.0, softness=0.5, erp=0.5, bounce=0.0):
        lib().orc_set_6dof_angular_motor(self.h, jid, axis, 1 if enable else 0, target_velocity, max_motor_force,
                                         max_limit_force, damping, softness, erp, bounce)

    def add_cone_twist(self, a, b, frame_a, frame_b):
        fa = np.ascontiguousarray(frame_a, np.float32).reshape(12)
        fb = np.ascontiguousarray(frame_b, np.float32).reshape(12)
        return lib().orc_add_cone_twist(self.h, a, b, _fp(fa), _fp(fb))

    def set_cone_limit(self, jid, swing1, swing2, twist, softness=0.8, bias_factor=0.3, relaxation_factor=1.0):
        lib().orc_set_cone_limit(self.h, jid, swing1, swing2, twist, softness, bias_factor, relaxation_factor)

    def add_slider(self, a, b, frame_a, frame_b, use_linear_reference_frame_a=True):
        fa = np.ascontiguousarray(frame_a, np.float32).reshape(12)
        fb = np.ascontiguousarray(frame_b, np.float32).reshape(12)
        return lib().orc_add_slider(self.h, a, b, _fp(fa), _fp(fb), 1 if use_linear_reference_frame_a else 0)

    def set_slider_params(self, jid, params):
        p = np.ascontiguousarray(params, np.float32).reshape(28)
        lib().orc_set_slider_params(self.h, jid, _fp(p))

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
                    self.set_hinge_angular_only(jid, True)
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
        return lib().orc_num_bodies(self.h)

    def set_ccd(self, bodies, motion_threshold, swept_sphere_radius):
        """CollisionObject.setCcdMotionThreshold / setCcdSweptSphereRadius for the given bodies."""
        b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
        t = np.ascontiguousarray(np.broadcast_to(np.float32(motion_threshold) if np.isscalar(motion_threshold)
                                                 else motion_threshold, b.shape), np.float32)
        r = np.ascontiguousarray(np.broadcast_to(np.float32(swept_sphere_radius) if np.isscalar(swept_sphere_radius)
                                                 else swept_sphere_radius, b.shape), np.float32)
        rc = lib().orc_set_ccd(self.h, b.ctypes.data_as(_abi.i32p), _fp(t), _fp(r), len(b))
        if rc != 0:
            raise ValueError("bad body index")

    def set_order_mode(self, mode):
        lib().orc_set_order_mode(self.h, mode)

    def set_explicit_order(self, order):
        o = np.ascontiguousarray(order, np.int32)
        lib().orc_set_explicit_order(self.h, o.ctypes.data_as(_abi.i32p), len(o))
        self.set_order_mode(ORDER_EXPLICIT)

    def set_brute_force_pairs(self, on=True):
        lib().orc_set_brute_force(self.h, 1 if on else 0)

    def step(self, dt, substeps=1):
        lib().orc_step(self.h, dt, substeps)
        if self._tick:
            self._tick.reraise()

    def step_simulation(self, time_step, max_sub_steps=1, fixed_time_step=1.0 / 60.0):
        n = lib().orc_step_simulation(self.h, time_step, max_sub_steps, fixed_time_step)
        if self._tick:
            self._tick.reraise()
        return n

    def set_internal_tick_callback(self, cb):
        """DynamicsWorld.setInternalTickCallback: cb(world, time_step) after every internal single step."""
        self._tick = None if cb is None else _abi.TickTrampoline(self, cb)
        lib().orc_set_tick_callback(self.h, _abi.TICK_CALLBACK() if self._tick is None else self._tick.fn, None)

    def set_body_properties(self, bodies, **props):
        """RigidBody.setDamping / setSleepingThresholds, CollisionObject.setFriction / setRestitution."""
        b, arrs = _abi.body_property_arrays(bodies, props)
        ptr = [None if a is None else _fp(a) for a in arrs]
        if lib().orc_set_body_properties(self.h, b.ctypes.data_as(_abi.i32p), len(b), *ptr) != 0:
            raise ValueError("set_body_properties: bad or repeated body index")

    def apply_impulses(self, bodies, impulses=None, rel_pos=None, torque_impulses=None):
        """RigidBody.applyCentralImpulse / applyImpulse (rel_pos given) / applyTorqueImpulse."""
        b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
        arrs = [None if a is None else np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float32).reshape(-1, 3),
                                                                            (len(b), 3)), np.float32)
                for a in (impulses, rel_pos, torque_impulses)]
        ptr = [None if a is None else _fp(a) for a in arrs]
        if lib().orc_apply_impulses(self.h, b.ctypes.data_as(_abi.i32p), ptr[0], ptr[1], ptr[2], len(b)) != 0:
            raise ValueError("apply_impulses: bad body index")

    def remove_bodies(self, bodies):
        """DiscreteDynamicsWorld.removeRigidBody for the given bodies (later bodies move down)."""
        b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
        if lib().orc_remove_bodies(self.h, b.ctypes.data_as(_abi.i32p), len(b)) != 0:
            raise ValueError("remove_bodies: bad index, repeated index or a body a joint uses")

    def set_gravity(self, g):
        """DiscreteDynamicsWorld.setGravity."""
        a = np.ascontiguousarray(g, np.float32).reshape(3)
        lib().orc_set_gravity(self.h, _fp(a))

    def set_body_gravity(self, bodies, acceleration):
        """RigidBody.setGravity for the given bodies (one acceleration each, or one for all)."""
        b = np.ascontiguousarray(bodies, np.int32).reshape(-1)
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(acceleration, np.float32).reshape(-1, 3), (len(b), 3)),
                                 np.float32)
        if lib().orc_set_body_gravity(self.h, b.ctypes.data_as(_abi.i32p), _fp(a), len(b)) != 0:
            raise ValueError("set_body_gravity: bad body index")

    def refit_mesh(self, shape, points):
        """New positions of a triangle mesh's vertices, then BvhTriangleMeshShape.refitTree and
        updateSingleAabb of its bodies."""
        p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        if lib().orc_refit_mesh(self.h, int(shape), _fp(p), len(p)) != 0:
            raise ValueError("refit_mesh: not a triangle mesh, or another vertex count")

    def mesh_bvh(self, shape):
        """The world's current tree of a triangle-mesh shape: (nodes (n, 4) int32, local aabb (6,))."""
        aabb = np.zeros(6, np.float32)
        n = lib().orc_world_mesh_bvh(self.h, int(shape), None, 0, _fp(aabb))
        if n < 0:
            raise ValueError("mesh_bvh: not a triangle mesh")
        nodes = np.zeros((n, 4), np.int32)
        lib().orc_world_mesh_bvh(self.h, int(shape), nodes.ctypes.data_as(_abi.i32p), n, _fp(aabb))
        return nodes, aabb

    def stage(self, stage, dt=1.0 / 60.0):
        lib().orc_stage(self.h, stage, dt)

    def get_state(self):
        sb = _abi.StateBuffers(self.n_bodies)
        lib().orc_get_state(self.h, C.byref(sb.struct))
        return sb.copy_arrays()

    def set_state(self, arrays):
        arrays = {k: v for k, v in arrays.items() if k != "island_tag"}
        sb = _abi.StateBuffers.from_arrays(arrays)
        rc = lib().orc_set_state(self.h, C.byref(sb.struct))
        assert rc == 0, rc

    def get_manifolds(self):
        cap = 1024
        while True:
            mb = _abi.ManifoldBuffers(cap)
            rc = lib().orc_get_manifolds(self.h, C.byref(mb.struct))
            if rc == 0:
                return mb.view()
            cap = mb.struct.n_pairs + 16

    def set_manifolds(self, m):
        mb = _abi.ManifoldBuffers.from_arrays(m["keys"], m["flags"], m["num_points"], m["points"])
        lib().orc_set_manifolds(self.h, C.byref(mb.struct))

    def get_pairs(self):
        return self.get_manifolds()["keys"]

    def solver_order(self):
        cap = max(16, self.counters()["pairs"] + 16)
        out = np.zeros(cap, np.int32)
        n = lib().orc_get_solver_order(self.h, out.ctypes.data_as(_abi.i32p), cap)
        return out[:n].copy()

    def counters(self):
        c = _abi.Counters()
        lib().orc_counters(self.h, C.byref(c))
        return c.as_dict()

    def phase_seconds(self):
        out = (C.c_double * 10)()
        lib().orc_phase_seconds(self.h, out)
        return list(out)


def shape_local_inertia(shape_dict, mass):
    from jbgpu.scenes import Scene
    sc = Scene("one", 0, 0, {}, [shape_dict], np.zeros(0))
    d = sc.shape_descs()
    out = np.zeros(3, np.float32)
    lib().orc_shape_local_inertia(C.byref(d[0]), mass, _fp(out))
    return out


def mesh_bvh(mesh_dict):
    """OptimizedBvh of a triangle-mesh shape dict as the oracle builds it: (nodes (n, 4) int32 in
    the library's layout, local aabb (6,))."""
    from jbgpu.scenes import shape_desc_array
    d = shape_desc_array([mesh_dict])
    nt = len(mesh_dict["indices"])
    nodes = np.zeros((2 * nt, 4), np.int32)
    aabb = np.zeros(6, np.float32)
    n = lib().orc_mesh_bvh(C.byref(d[0]), nodes.ctypes.data_as(_abi.i32p), len(nodes), _fp(aabb))
    return nodes[:n].copy(), aabb


def mesh_query(mesh_dict, aabb_min, aabb_max):
    """OptimizedBvh.reportAabbOverlappingNodex: triangle indices in report order."""
    from jbgpu.scenes import shape_desc_array
    d = shape_desc_array([mesh_dict])
    mn = np.ascontiguousarray(aabb_min, np.float32)
    mx = np.ascontiguousarray(aabb_max, np.float32)
    out = np.zeros(len(mesh_dict["indices"]), np.int32)
    n = lib().orc_mesh_query(C.byref(d[0]), _fp(mn), _fp(mx), out.ctypes.data_as(_abi.i32p), len(out))
    return out[:n].copy()


def gjk(shape_a, xf_a, shape_b, xf_b, max_dist2):
    from jbgpu.scenes import Scene
    sc = Scene("two", 0, 0, {}, [shape_a, shape_b], np.zeros(0))
    d = sc.shape_descs()
    ta = np.ascontiguousarray(xf_a, np.float32)
    tb = np.ascontiguousarray(xf_b, np.float32)
    out = np.zeros(9, np.float32)
    lib().orc_gjk(C.byref(d[0]), _fp(ta), C.byref(d[1]), _fp(tb), max_dist2, _fp(out))
    return out


def integrate_transform(t12, lin, ang, dt):
    t = np.ascontiguousarray(t12, np.float32)
    l = np.ascontiguousarray(lin, np.float32)
    a = np.ascontiguousarray(ang, np.float32)
    out = np.zeros(12, np.float32)
    lib().orc_integrate_transform(_fp(t), _fp(l), _fp(a), dt, _fp(out))
    return out
