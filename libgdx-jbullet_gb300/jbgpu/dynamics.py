"""Host-side mirror of the reference's world / body / shape API over the C ABI.

Names, argument meaning and defaults follow JBullet (src/com/bulletphysics/ of the reference):
DiscreteDynamicsWorld (dynamics/DiscreteDynamicsWorld.java), RigidBody and
RigidBodyConstructionInfo (dynamics/RigidBody.java, RigidBodyConstructionInfo.java), the
shapes of collision/shapes/, ContactSolverInfo (dynamics/constraintsolver/ContactSolverInfo.java).
The dispatcher, broadphase and constraint solver arguments of the world constructor are
accepted and ignored: the GPU step replaces all three behind the same stepSimulation call.

Bodies are staged on the host and uploaded in bulk the first time the world steps (or when
queried); after that their state lives on the device and RigidBody getters read it back.
"""
import numpy as np

from . import _abi
from .lib import GpuWorld

ACTIVE_TAG, ISLAND_SLEEPING, WANTS_DEACTIVATION, DISABLE_DEACTIVATION, DISABLE_SIMULATION = 1, 2, 3, 4, 5


class Transform:
    """linearmath/Transform.java: basis (3x3, row-major) and origin."""

    def __init__(self, basis=None, origin=(0.0, 0.0, 0.0)):
        self.basis = np.eye(3, dtype=np.float32) if basis is None else np.asarray(basis, np.float32).reshape(3, 3)
        self.origin = np.asarray(origin, np.float32).reshape(3)

    def setIdentity(self):
        self.basis = np.eye(3, dtype=np.float32)
        self.origin = np.zeros(3, np.float32)

    def as12(self):
        return np.concatenate([self.basis.reshape(9), self.origin]).astype(np.float32)

    @classmethod
    def from12(cls, t):
        return cls(np.asarray(t[:9]).reshape(3, 3), t[9:12])


F32 = np.float32


def _crs(a, b):
    """Vector3.crs in binary32: a x b."""
    a = np.asarray(a, F32).reshape(3)
    b = np.asarray(b, F32).reshape(3)
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], F32)


def _clamp01(x):
    """MiscUtil.GEN_clamped(x, 0, 1) in binary32."""
    x = F32(x)
    return F32(0.0) if x < F32(0.0) else (F32(1.0) if F32(1.0) < x else x)


def _quat_from_basis(m):
    """RigidBody.getOrientation: MatrixUtil.getRotation, i.e. libGDX Quaternion.setFromMatrix(true, basis)
    (rows normalised, then the trace or largest-diagonal branch, the "1 + ..." sums in double);
    returns (x, y, z, w) as binary32."""
    m = np.asarray(m, F32).reshape(3, 3)
    r = [m[i] * (F32(1.0) / F32(np.sqrt(float(m[i, 0] * m[i, 0] + m[i, 1] * m[i, 1] + m[i, 2] * m[i, 2]))))
         for i in range(3)]
    (xx, xy, xz), (yx, yy, yz), (zx, zy, zz) = r
    t = xx + yy + zz
    half = F32(0.5)
    if t >= 0:
        sq = F32(np.sqrt(float(t + F32(1.0))))
        w = half * sq
        k = half / sq
        return np.array([(zy - yz) * k, (xz - zx) * k, (yx - xy) * k, w], F32)
    if xx > yy and xx > zz:
        sq = F32(np.sqrt(1.0 + float(xx) - float(yy) - float(zz)))
        k = half / sq
        return np.array([sq * half, (yx + xy) * k, (xz + zx) * k, (zy - yz) * k], F32)
    if yy > zz:
        sq = F32(np.sqrt(1.0 + float(yy) - float(xx) - float(zz)))
        k = half / sq
        return np.array([(yx + xy) * k, sq * half, (zy + yz) * k, (xz - zx) * k], F32)
    sq = F32(np.sqrt(1.0 + float(zz) - float(xx) - float(yy)))
    k = half / sq
    return np.array([(xz + zx) * k, (zy + yz) * k, sq * half, (yx - xy) * k], F32)


class _Shape:
    shape_type = None

    def __init__(self):
        self._id = None

    def desc(self):
        raise NotImplementedError

    def calculateLocalInertia(self, mass):
        """CollisionShape.calculateLocalInertia (binary32, the reference's operation order)."""
        from . import lib
        return lib.shape_local_inertia(self.desc(), mass)


class BoxShape(_Shape):
    def __init__(self, boxHalfExtents):
        super().__init__()
        self.halfExtents = tuple(float(x) for x in boxHalfExtents)

    def desc(self):
        return {"type": _abi.SHAPE_BOX, "params": self.halfExtents + (0.0,), "points": None}


class SphereShape(_Shape):
    def __init__(self, radius):
        super().__init__()
        self.radius = float(radius)

    def desc(self):
        return {"type": _abi.SHAPE_SPHERE, "params": (self.radius, 0.0, 0.0, 0.0), "points": None}


class CapsuleShape(_Shape):
    def __init__(self, radius, height):
        super().__init__()
        self.radius, self.height = float(radius), float(height)

    def desc(self):
        return {"type": _abi.SHAPE_CAPSULE, "params": (self.radius, self.height, 0.0, 0.0), "points": None}


class ConvexHullShape(_Shape):
    def __init__(self, points):
        super().__init__()
        self.points = np.asarray(points, np.float32).reshape(-1, 3)

    def desc(self):
        return {"type": _abi.SHAPE_CONVEX_HULL, "params": (0.0, 0.0, 0.0, 0.0), "points": self.points}


class StaticPlaneShape(_Shape):
    def __init__(self, planeNormal, planeConstant):
        super().__init__()
        self.normal, self.constant = tuple(float(x) for x in planeNormal), float(planeConstant)

    def desc(self):
        return {"type": _abi.SHAPE_STATIC_PLANE, "params": self.normal + (self.constant,), "points": None}


class TriangleIndexVertexArray:
    """collision/shapes/TriangleIndexVertexArray.java with one IndexedMesh part: triangle vertex
    indices (m, 3) and vertices (n, 3); its scaling is set through BvhTriangleMeshShape.setLocalScaling."""

    def __init__(self, triangleIndices, vertices):
        self.indices = np.ascontiguousarray(triangleIndices, np.int32).reshape(-1, 3)
        self.vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)

    def getNumSubParts(self):
        return 1


class BvhTriangleMeshShape(_Shape):
    """collision/shapes/BvhTriangleMeshShape.java over a TriangleIndexVertexArray, with the
    quantized OptimizedBvh (useQuantizedAabbCompression = true, the tree the library builds and
    walks).  For static (mass 0) or kinematic bodies, as in the reference."""

    def __init__(self, meshInterface, useQuantizedAabbCompression=True):
        super().__init__()
        if not useQuantizedAabbCompression:
            raise NotImplementedError("only the quantized tree (useQuantizedAabbCompression=True) is built")
        self.meshInterface = meshInterface
        self.margin = 0.0   # ConcaveShape.collisionMargin
        self.scaling = (0.0, 0.0, 0.0)   # (0, 0, 0): setLocalScaling not called

    def setMargin(self, margin):
        if self._id is not None:
            raise RuntimeError("setMargin after the shape was added to a world")
        self.margin = float(margin)

    def setLocalScaling(self, scaling):
        """BvhTriangleMeshShape.setLocalScaling (java:195-212): the tree is rebuilt over the scaled
        vertices.  Its quantization bounds then include the margin set so far, so only a call
        before setMargin is supported."""
        if self._id is not None:
            raise RuntimeError("setLocalScaling after the shape was added to a world")
        if self.margin != 0.0:
            raise NotImplementedError("setLocalScaling after setMargin (the rebuilt tree's bounds would include the margin)")
        self.scaling = tuple(float(x) for x in scaling)

    def getLocalScaling(self):
        s = self.scaling
        d = np.float32(1.0) - np.asarray(s, np.float32)
        if s == (0.0, 0.0, 0.0) or not (np.float32(d[0] * d[0] + d[1] * d[1]) + np.float32(d[2] * d[2]) > np.float32(1.1920929e-7)):
            return np.ones(3, np.float32)
        return np.asarray(s, np.float32)

    def getMargin(self):
        return self.margin

    def getMeshInterface(self):
        return self.meshInterface

    def refitTree(self, aabbMin=None, aabbMax=None):
        """BvhTriangleMeshShape.refitTree (java:172-178) after meshInterface.vertices were changed
        in place (same count): the tree is refitted and, as CollisionWorld.updateSingleAabb would
        be called for them, the aabbs of the bodies using the shape are recomputed.  The shape
        must have been added to a world (the world's tree is the one refitted)."""
        if self._id is None or getattr(self, "_world", None) is None or self._world._g is None:
            raise RuntimeError("refitTree on a shape that is not in a world yet")
        self._world._g.refit_mesh(self._id, self.meshInterface.vertices)

    def desc(self):
        return {"type": _abi.SHAPE_TRIANGLE_MESH, "params": (self.margin,) + self.scaling,
                "points": self.meshInterface.vertices, "indices": self.meshInterface.indices}

    def calculateLocalInertia(self, mass):
        return np.zeros(3, np.float32)   # TriangleMeshShape.calculateLocalInertia: moving meshes unsupported


class CompoundShape(_Shape):
    """collision/shapes/CompoundShape.java: convex children (boxes, spheres, capsules, convex
    hulls) at local transforms, at most 16 of them; collisionMargin 0."""

    def __init__(self):
        super().__init__()
        self.children = []
        self.margin = 0.0

    def addChildShape(self, localTransform, shape):
        if self._id is not None:
            raise RuntimeError("addChildShape after the shape was added to a world")
        if len(self.children) >= _abi.COMPOUND_MAX_CHILDREN:
            raise ValueError("a compound holds at most %d children" % _abi.COMPOUND_MAX_CHILDREN)
        if isinstance(shape, (CompoundShape, BvhTriangleMeshShape, StaticPlaneShape)):
            raise NotImplementedError("compound children must be convex shapes")
        self.children.append((Transform(localTransform.basis.copy(), localTransform.origin.copy()), shape))

    def getNumChildShapes(self):
        return len(self.children)

    def getChildShape(self, i):
        return self.children[i][1]

    def getChildTransform(self, i):
        t = self.children[i][0]
        return Transform(t.basis.copy(), t.origin.copy())

    def setMargin(self, margin):
        if self._id is not None:
            raise RuntimeError("setMargin after the shape was added to a world")
        self.margin = float(margin)

    def getMargin(self):
        return self.margin

    def desc(self):
        return {"type": _abi.SHAPE_COMPOUND, "params": (self.margin, 0.0, 0.0, 0.0), "points": None,
                "children": [(s.desc(), t.as12()) for t, s in self.children]}


class RigidBodyConstructionInfo:
    def __init__(self, mass, motionState, collisionShape, localInertia=(0.0, 0.0, 0.0)):
        self.mass = float(mass)
        self.motionState = motionState
        self.collisionShape = collisionShape
        self.localInertia = tuple(float(x) for x in localInertia)
        self.startWorldTransform = Transform()
        self.linearDamping = 0.0
        self.angularDamping = 0.0
        self.friction = 0.5
        self.restitution = 0.0
        self.linearSleepingThreshold = 0.8
        self.angularSleepingThreshold = 1.0


class RigidBody:
    def __init__(self, info):
        self.info = info
        self._world = None
        self._index = None
        self._linvel = (0.0, 0.0, 0.0)
        self._angvel = (0.0, 0.0, 0.0)
        self._group = -1
        self._mask = -1
        self._ccd = (0.0, 0.0)          # ccdMotionThreshold, ccdSweptSphereRadius
        self._flags = 0                 # KINEMATIC_OBJECT / NO_CONTACT_RESPONSE set before addRigidBody
        self._activation = 0            # setActivationState before addRigidBody (0: ACTIVE_TAG)
        self._gravity_acc = None        # RigidBody.setGravity staged until the body is on the device

    def setGravity(self, acceleration):
        """RigidBody.setGravity (RigidBody.java:213-217).  Before addRigidBody it has no lasting
        effect: addRigidBody sets the world's gravity on a body that is not static or kinematic."""
        a = tuple(float(x) for x in acceleration)
        if self._world is None:
            return
        if self._world._g is not None and self._index < self._world._uploaded:
            self._world._g.set_body_gravity([self._index], [a])
        else:
            self._gravity_acc = a

    # CollisionObject.setCollisionFlags / getCollisionFlags (collision/dispatch/CollisionObject.java):
    # KINEMATIC_OBJECT and NO_CONTACT_RESPONSE, set before the body is added; STATIC_OBJECT
    # follows from mass 0
    def setCollisionFlags(self, flags):
        if self._world is not None:
            raise NotImplementedError("setCollisionFlags after addRigidBody")
        if flags & ~(_abi.CF_STATIC_OBJECT | _abi.CF_KINEMATIC_OBJECT | _abi.CF_NO_CONTACT_RESPONSE):
            raise NotImplementedError("collision flags other than KINEMATIC_OBJECT and NO_CONTACT_RESPONSE")
        self._flags = int(flags) & (_abi.CF_KINEMATIC_OBJECT | _abi.CF_NO_CONTACT_RESPONSE)

    def getCollisionFlags(self):
        return self._flags | (_abi.CF_STATIC_OBJECT if self.info.mass == 0.0 else 0)

    def isKinematicObject(self):
        return (self._flags & _abi.CF_KINEMATIC_OBJECT) != 0

    def setActivationState(self, state):
        """CollisionObject.setActivationState: no change from DISABLE_DEACTIVATION or DISABLE_SIMULATION."""
        if self._world is None or self._world._g is None:
            if self._activation not in (DISABLE_DEACTIVATION, DISABLE_SIMULATION):
                self._activation = int(state)
            return
        if self.getActivationState() not in (DISABLE_DEACTIVATION, DISABLE_SIMULATION):
            self._world._set_field("activation_state", self._index, int(state))

    def forceActivationState(self, state):
        if self._world is None or self._world._g is None:
            self._activation = int(state)
        else:
            self._world._set_field("activation_state", self._index, int(state))

    def setWorldTransform(self, transform):
        """CollisionObject.setWorldTransform: for a kinematic body, the pose saveKinematicState
        turns into velocities at the next stepSimulation."""
        if self._world is not None and self._world._g is not None:
            self._world._set_field("transform", self._index, transform.as12())
        else:
            self.info.startWorldTransform = transform

    # velocities set before the body enters the world are uploaded with it
    def setLinearVelocity(self, v):
        if self._world is not None and self._world._g is not None:
            self._world._set_field("linear_velocity", self._index, v)
        else:
            self._linvel = tuple(float(x) for x in v)

    def setAngularVelocity(self, v):
        if self._world is not None and self._world._g is not None:
            self._world._set_field("angular_velocity", self._index, v)
        else:
            self._angvel = tuple(float(x) for x in v)

    def _state(self, field):
        return self._world._get_field(field, self._index)

    def getCenterOfMassTransform(self):
        return Transform.from12(self._state("transform"))

    getWorldTransform = getCenterOfMassTransform

    def getLinearVelocity(self):
        return self._state("linear_velocity")

    def getAngularVelocity(self):
        return self._state("angular_velocity")

    def getActivationState(self):
        return int(self._state("activation_state"))

    def isActive(self):
        return self.getActivationState() not in (ISLAND_SLEEPING, DISABLE_SIMULATION)

    def getInvMass(self):
        return 0.0 if self.info.mass == 0.0 else 1.0 / np.float32(self.info.mass)

    def applyCentralForce(self, f):
        self._world._pending_force(self._index, force=f)

    # RigidBody.applyTorque / applyForce / clearForces (RigidBody.java:355-394): the accumulators
    # totalForce / totalTorque that stepSimulation's substeps integrate and then clear
    def applyTorque(self, torque):
        self._world._pending_force(self._index, torque=torque)

    def applyForce(self, force, rel_pos):
        self.applyCentralForce(force)
        self.applyTorque(_crs(rel_pos, force))

    def clearForces(self):
        w = self._world
        if w is None:
            return
        w._flush_forces()
        if w._g is not None:
            st = w._state()
            st["total_force"][self._index] = 0.0
            st["total_torque"][self._index] = 0.0
            w._g.set_state({"total_force": st["total_force"], "total_torque": st["total_torque"]})
            w._cache = None

    def getTotalForce(self):
        self._world._flush_forces()
        return self._state("total_force")

    def getTotalTorque(self):
        self._world._flush_forces()
        return self._state("total_torque")

    # per-body properties (RigidBody.java:224-227, 371-374; CollisionObject.java:186-196): kept
    # in the construction info until the body is on the device, written there after
    def _live(self):
        return self._world is not None and self._world._g is not None and self._index < self._world._uploaded

    def _set_props(self, **kw):
        if self._live():
            self._world._g.set_body_properties([self._index], **kw)

    def setDamping(self, lin_damping, ang_damping):
        self.info.linearDamping = float(_clamp01(lin_damping))
        self.info.angularDamping = float(_clamp01(ang_damping))
        self._set_props(linear_damping=lin_damping, angular_damping=ang_damping)

    def getLinearDamping(self):
        return float(_clamp01(self.info.linearDamping))

    def getAngularDamping(self):
        return float(_clamp01(self.info.angularDamping))

    def setFriction(self, friction):
        self.info.friction = float(friction)
        self._set_props(friction=friction)

    def getFriction(self):
        return self.info.friction

    def setRestitution(self, restitution):
        self.info.restitution = float(restitution)
        self._set_props(restitution=restitution)

    def getRestitution(self):
        return self.info.restitution

    def setSleepingThresholds(self, linear, angular):
        self.info.linearSleepingThreshold = float(linear)
        self.info.angularSleepingThreshold = float(angular)
        self._set_props(linear_sleeping_threshold=linear, angular_sleeping_threshold=angular)

    def getLinearSleepingThreshold(self):
        return self.info.linearSleepingThreshold

    def getAngularSleepingThreshold(self):
        return self.info.angularSleepingThreshold

    def getLinearFactor(self):
        return np.ones(3, F32)

    def getAngularFactor(self):
        return np.ones(3, F32)

    # CollisionObject / RigidBody getters over the body's device state
    def getCollisionShape(self):
        return self.info.collisionShape

    def getMotionState(self):
        return self.info.motionState

    def setMotionState(self, motionState):
        self.info.motionState = motionState

    def isInWorld(self):
        return self._world is not None

    _user = None

    def getUserPointer(self):
        return self._user

    def setUserPointer(self, obj):
        self._user = obj

    def isStaticObject(self):
        return (self.getCollisionFlags() & _abi.CF_STATIC_OBJECT) != 0

    def isStaticOrKinematicObject(self):
        return (self.getCollisionFlags() & (_abi.CF_STATIC_OBJECT | _abi.CF_KINEMATIC_OBJECT)) != 0

    def hasContactResponse(self):
        return (self.getCollisionFlags() & _abi.CF_NO_CONTACT_RESPONSE) == 0

    def mergesSimulationIslands(self):
        return (self.getCollisionFlags() & (_abi.CF_STATIC_OBJECT | _abi.CF_KINEMATIC_OBJECT |
                                            _abi.CF_NO_CONTACT_RESPONSE)) == 0

    def getCenterOfMassPosition(self):
        return self._state("transform")[9:12].copy()

    def getOrientation(self):
        return _quat_from_basis(self._state("transform")[:9])

    def getVelocityInLocalPoint(self, rel_pos):
        """RigidBody.getVelocityInLocalPoint: linearVelocity + angularVelocity x rel_pos."""
        return (self.getLinearVelocity() + _crs(self.getAngularVelocity(), rel_pos)).astype(F32)

    def getInvInertiaTensorWorld(self):
        return self._state("inv_inertia_world").reshape(3, 3).copy()

    def getInvInertiaDiagLocal(self):
        """RigidBody.setMassProps: 1 / localInertia per axis, 0 where it is 0."""
        li = np.asarray(self.info.localInertia, F32)
        return np.array([F32(0.0) if x == 0.0 else F32(1.0) / x for x in li], F32)

    def getAabb(self):
        a = self._state("aabb")
        return a[:3].copy(), a[3:].copy()

    def getIslandTag(self):
        return int(self._state("island_tag"))

    def getDeactivationTime(self):
        return float(self._state("deactivation_time"))

    def setDeactivationTime(self, t):
        if self._world is None or self._world._g is None:
            raise RuntimeError("setDeactivationTime applies to a body in a world that has stepped")
        self._world._set_field("deactivation_time", self._index, float(t))

    def activate(self, forceActivation=False):
        """CollisionObject.activate: ACTIVE_TAG and deactivationTime 0 unless the body is static or
        kinematic (and forceActivation is false)."""
        if forceActivation or not self.isStaticOrKinematicObject():
            self.setActivationState(ACTIVE_TAG)
            if self._world is not None and self._world._g is not None:
                self._world._set_field("deactivation_time", self._index, 0.0)

    # RigidBody.applyCentralImpulse / applyImpulse / applyTorqueImpulse (RigidBody.java:395-430):
    # the velocity changes now, on the body's device state (the body must be in a world)
    def _impulse(self, **kw):
        if self._world is None:
            raise RuntimeError("impulses apply to a body added to a DiscreteDynamicsWorld")
        self._world._ensure().apply_impulses([self._index], **kw)
        self._world._cache = None

    def applyCentralImpulse(self, impulse):
        self._impulse(impulses=[impulse])

    def applyImpulse(self, impulse, rel_pos):
        self._impulse(impulses=[impulse], rel_pos=[rel_pos])

    def applyTorqueImpulse(self, torque):
        self._impulse(torque_impulses=[torque])

    def getUid(self):
        return self._index + 1

    # CollisionObject.setCcdMotionThreshold / setCcdSweptSphereRadius (collision/dispatch/
    # CollisionObject.java:278-300): read by integrateTransforms' CCD motion clamping
    def setCcdMotionThreshold(self, t):
        self._ccd = (float(t), self._ccd[1])
        self._push_ccd()

    def setCcdSweptSphereRadius(self, r):
        self._ccd = (self._ccd[0], float(r))
        self._push_ccd()

    def getCcdMotionThreshold(self):
        return self._ccd[0]

    def getCcdSquareMotionThreshold(self):
        return float(np.float32(self._ccd[0]) * np.float32(self._ccd[0]))

    def getCcdSweptSphereRadius(self):
        return self._ccd[1]

    def _push_ccd(self):
        if self._world is not None and self._world._g is not None and self._index < self._world._uploaded:
            self._world._g.set_ccd([self._index], self._ccd[0], self._ccd[1])


class ContactSolverInfo:
    def __init__(self):
        self.numIterations = 10
        self.erp = 0.2
        self.warmstartingFactor = 0.85
        self.linearSlop = 0.0
        self.solverMode = _abi.SOLVER_CACHE_FRIENDLY | _abi.SOLVER_USE_WARMSTARTING


class ConstraintSetting:
    """Point2PointConstraint.ConstraintSetting (Point2PointConstraint.java:202-206)."""

    def __init__(self):
        self.tau = 0.3
        self.damping = 1.0
        self.impulseClamp = 0.0


class Point2PointConstraint:
    """dynamics/constraintsolver/Point2PointConstraint.java:37-70: Point2PointConstraint(rbA, rbB,
    pivotInA, pivotInB), or Point2PointConstraint(rbA, pivotInA) joining rbA to the fixed body at
    pivotInA taken to world space by rbA's current transform."""

    def __init__(self, rbA, *args):
        self.rbA = rbA
        if len(args) == 1:
            self.rbB = None
            self.pivotInA = np.asarray(args[0], np.float32)
            t = rbA.getCenterOfMassTransform()
            self.pivotInB = (t.basis @ self.pivotInA + t.origin).astype(np.float32)
        else:
            self.rbB, pa, pb = args
            self.pivotInA = np.asarray(pa, np.float32)
            self.pivotInB = np.asarray(pb, np.float32)
        self.setting = ConstraintSetting()
        self._world = None
        self._id = None

    def getRigidBodyA(self):
        return self.rbA

    def getRigidBodyB(self):
        return self.rbB

    def getPivotInA(self):
        return self.pivotInA.copy()

    def getPivotInB(self):
        return self.pivotInB.copy()

    def getAppliedImpulse(self):
        """TypedConstraint.getAppliedImpulse: the impulse of the last solve."""
        if self._world is None or self._world._g is None:
            return 0.0
        return float(self._world._g.joint_impulses()[self._id])


class HingeConstraint:
    """dynamics/constraintsolver/HingeConstraint.java:44-620, with its four constructors:
    HingeConstraint(rbA, rbB, pivotInA, pivotInB, axisInA, axisInB), HingeConstraint(rbA,
    pivotInA, axisInA), HingeConstraint(rbA, rbB, rbAFrame, rbBFrame) and HingeConstraint(rbA,
    rbAFrame) (frames as Transform).  The frames are computed as the reference's constructors
    compute them (jbgpu.frames) from the bodies' transforms at construction."""

    def __init__(self, rbA, *args):
        from . import frames
        self.rbA = rbA
        ta = rbA.getCenterOfMassTransform()
        if len(args) == 5:
            self.rbB, pa, pb, axa, axb = args
            fa, fb = frames.hinge_frames_two_bodies(ta.basis, pa, pb, axa, axb)
        elif len(args) == 2 and not isinstance(args[0], Transform):
            self.rbB = None
            fa, fb = frames.hinge_frames_one_body(ta.as12(), args[0], args[1])
        elif len(args) == 3:
            self.rbB = args[0]
            fa, fb = frames.hinge_frames_from_frames(ta.as12(), args[1].as12(), args[2].as12())
        elif len(args) == 1:
            self.rbB = None
            fa, fb = frames.hinge_frames_from_frames(ta.as12(), args[0].as12())
        else:
            raise TypeError("HingeConstraint(rbA, rbB, pivotInA, pivotInB, axisInA, axisInB), (rbA, pivotInA, axisInA), "
                            "(rbA, rbB, rbAFrame, rbBFrame) or (rbA, rbAFrame)")
        self.frameA, self.frameB = Transform.from12(fa), Transform.from12(fb)
        self.lowerLimit, self.upperLimit = 1e30, -1e30
        self.limitSoftness, self.biasFactor, self.relaxationFactor = 0.9, 0.3, 1.0
        self.angularOnly = False
        self.enableMotor, self.motorTargetVelocity, self.maxMotorImpulse = False, 0.0, 0.0
        self._world = None
        self._id = None

    def _push(self):
        g = self._world._g if self._world is not None else None
        if g is None or self._id is None:
            return
        g.set_hinge_limit(self._id, self.lowerLimit, self.upperLimit, self.limitSoftness, self.biasFactor,
                          self.relaxationFactor)
        g.enable_hinge_motor(self._id, self.enableMotor, self.motorTargetVelocity, self.maxMotorImpulse)
        g.set_hinge_angular_only(self._id, self.angularOnly)

    def setLimit(self, low, high, softness=0.9, biasFactor=0.3, relaxationFactor=1.0):
        self.lowerLimit, self.upperLimit = float(low), float(high)
        self.limitSoftness, self.biasFactor, self.relaxationFactor = float(softness), float(biasFactor), float(relaxationFactor)
        self._push()

    def enableAngularMotor(self, enableMotor, targetVelocity, maxMotorImpulse):
        self.enableMotor = bool(enableMotor)
        self.motorTargetVelocity, self.maxMotorImpulse = float(targetVelocity), float(maxMotorImpulse)
        self._push()

    def setAngularOnly(self, angularOnly):
        self.angularOnly = bool(angularOnly)
        self._push()

    def getRigidBodyA(self):
        return self.rbA

    def getRigidBodyB(self):
        return self.rbB

    def getAFrame(self):
        return Transform(self.frameA.basis.copy(), self.frameA.origin.copy())

    def getBFrame(self):
        return Transform(self.frameB.basis.copy(), self.frameB.origin.copy())

    def getLowerLimit(self):
        return self.lowerLimit

    def getUpperLimit(self):
        return self.upperLimit

    def getAngularOnly(self):
        return self.angularOnly

    def getEnableAngularMotor(self):
        return self.enableMotor

    def getMaxMotorImpulse(self):
        return self.maxMotorImpulse

    def getHingeAngle(self):
        """HingeConstraint.getHingeAngle (java:535-555) from the bodies' current transforms,
        with ScalarUtil.atan2Fast, in binary32."""
        from . import frames
        F = np.float32
        ta = self.rbA.getCenterOfMassTransform()
        tb = self.rbB.getCenterOfMassTransform() if self.rbB is not None else Transform()
        ref0 = frames._mulMv(ta.basis, frames._col(self.frameA.basis, 0))
        ref1 = frames._mulMv(ta.basis, frames._col(self.frameA.basis, 1))
        swing = frames._mulMv(tb.basis, frames._col(self.frameB.basis, 1))
        y, x = frames._dot(swing, ref0), frames._dot(swing, ref1)
        c1 = F(F(6.283185307179586232) * F(0.5)) / F(4.0)
        c2 = F(3.0) * c1
        ay = abs(y)
        angle = c1 - c1 * ((x - ay) / (x + ay)) if x >= 0 else c2 - c1 * ((x + ay) / (ay - x))
        return float(-angle if y < 0 else angle)

    def getAppliedImpulse(self):
        """TypedConstraint.getAppliedImpulse: the sum of the linear rows' impulses of the last solve."""
        if self._world is None or self._world._g is None:
            return 0.0
        return float(self._world._g.joint_impulses()[self._id])


class ConeTwistConstraint:
    """dynamics/constraintsolver/ConeTwistConstraint.java:43-412: ConeTwistConstraint(rbA, rbB,
    rbAFrame, rbBFrame) or ConeTwistConstraint(rbA, rbAFrame) (B's frame = A's frame, unchanged, on
    the fixed body, as the reference's constructor leaves it)."""

    def __init__(self, rbA, *args):
        self.rbA = rbA
        if len(args) == 3:
            self.rbB, fa, fb = args
        else:
            self.rbB, fa, fb = None, args[0], args[0]
        self.frameA = Transform(fa.basis.copy(), fa.origin.copy())
        self.frameB = Transform(fb.basis.copy(), fb.origin.copy())
        self.swingSpan1 = self.swingSpan2 = self.twistSpan = 1e30
        self.limitSoftness, self.biasFactor, self.relaxationFactor = 0.0, 0.3, 1.0
        self.angularOnly = False
        self._world = None
        self._id = None

    def _push(self):
        g = self._world._g if self._world is not None else None
        if g is None or self._id is None:
            return
        g.set_cone_limit(self._id, self.swingSpan1, self.swingSpan2, self.twistSpan, self.limitSoftness, self.biasFactor,
                         self.relaxationFactor)
        g.set_cone_angular_only(self._id, self.angularOnly)

    def setLimit(self, swingSpan1, swingSpan2, twistSpan, softness=0.8, biasFactor=0.3, relaxationFactor=1.0):
        self.swingSpan1, self.swingSpan2, self.twistSpan = float(swingSpan1), float(swingSpan2), float(twistSpan)
        self.limitSoftness, self.biasFactor, self.relaxationFactor = float(softness), float(biasFactor), float(relaxationFactor)
        self._push()

    def setAngularOnly(self, angularOnly):
        self.angularOnly = bool(angularOnly)
        self._push()

    def getRigidBodyA(self):
        return self.rbA

    def getRigidBodyB(self):
        return self.rbB

    def getAFrame(self):
        return Transform(self.frameA.basis.copy(), self.frameA.origin.copy())

    def getBFrame(self):
        return Transform(self.frameB.basis.copy(), self.frameB.origin.copy())

    def getAppliedImpulse(self):
        if self._world is None or self._world._g is None:
            return 0.0
        return float(self._world._g.joint_impulses()[self._id])


class SliderConstraint:
    """dynamics/constraintsolver/SliderConstraint.java:130-685: SliderConstraint(rbA, rbB, frameInA,
    frameInB, useLinearReferenceFrameA) with the reference's setters (limits, the softness /
    restitution / damping of its six row groups, the two motors); changes are sent before the
    next step."""

    _names = ["LowerLinLimit", "UpperLinLimit", "LowerAngLimit", "UpperAngLimit"]
    for _g in ("DirLin", "DirAng", "LimLin", "LimAng", "OrthoLin", "OrthoAng"):
        _names += ["Softness" + _g, "Restitution" + _g, "Damping" + _g]
    _names += ["PoweredLinMotor", "TargetLinMotorVelocity", "MaxLinMotorForce", "PoweredAngMotor",
               "TargetAngMotorVelocity", "MaxAngMotorForce"]

    def __init__(self, rbA, rbB, frameInA, frameInB, useLinearReferenceFrameA):
        self.rbA, self.rbB = rbA, rbB
        self.frameInA = Transform(frameInA.basis.copy(), frameInA.origin.copy())
        self.frameInB = Transform(frameInB.basis.copy(), frameInB.origin.copy())
        self.useLinearReferenceFrameA = bool(useLinearReferenceFrameA)
        self.params = np.array([1.0, -1.0, 0.0, 0.0] + [1.0, 0.7, 0.0] * 2 + [1.0, 0.7, 1.0] * 4 + [0.0] * 6, np.float32)
        self._world = None
        self._id = None
        self._sent = None

    def __getattr__(self, name):
        for prefix in ("set", "get"):
            if name.startswith(prefix) and name[3:] in SliderConstraint._names:
                k = SliderConstraint._names.index(name[3:])
                if prefix == "set":
                    return lambda v: self.params.__setitem__(k, float(v))
                return lambda: (bool(self.params[k]) if name[3:].startswith("Powered") else float(self.params[k]))
        raise AttributeError(name)

    def _push(self):
        g = self._world._g if self._world is not None else None
        if g is None or self._id is None:
            return
        if self._sent is not None and np.array_equal(self._sent, self.params):
            return
        g.set_slider_params(self._id, self.params)
        self._sent = self.params.copy()

    def getRigidBodyA(self):
        return self.rbA

    def getRigidBodyB(self):
        return self.rbB

    def getAppliedImpulse(self):
        return 0.0    # the reference's slider leaves TypedConstraint.appliedImpulse at 0


class RotationalLimitMotor:
    """dynamics/constraintsolver/RotationalLimitMotor.java:44-70 (settings; defaults as there)."""

    def __init__(self):
        self.loLimit, self.hiLimit = -3.40282347e+38, 3.40282347e+38
        self.targetVelocity, self.maxMotorForce, self.maxLimitForce = 0.0, 0.1, 300.0
        self.damping, self.limitSoftness, self.ERP, self.bounce = 1.0, 0.5, 0.5, 0.0
        self.enableMotor = False


class TranslationalLimitMotor:
    """dynamics/constraintsolver/TranslationalLimitMotor.java:38-56 (settings; defaults as there)."""

    def __init__(self):
        self.lowerLimit = np.zeros(3, np.float32)
        self.upperLimit = np.zeros(3, np.float32)
        self.limitSoftness, self.damping, self.restitution = 0.7, 1.0, 0.5


class Generic6DofConstraint:
    """dynamics/constraintsolver/Generic6DofConstraint.java:88-490: Generic6DofConstraint(rbA, rbB,
    frameInA, frameInB, useLinearReferenceFrameA) with its limit motors; settings changed after
    the constraint entered the world are sent before the next step."""

    def __init__(self, rbA, rbB, frameInA, frameInB, useLinearReferenceFrameA):
        self.rbA, self.rbB = rbA, rbB
        self.frameInA = Transform(frameInA.basis.copy(), frameInA.origin.copy())
        self.frameInB = Transform(frameInB.basis.copy(), frameInB.origin.copy())
        self.useLinearReferenceFrameA = bool(useLinearReferenceFrameA)
        self.linearLimits = TranslationalLimitMotor()
        self.angularLimits = [RotationalLimitMotor() for _ in range(3)]
        self._world = None
        self._id = None
        self._sent = None

    def setLimit(self, axis, lo, hi):
        if axis < 3:
            self.linearLimits.lowerLimit[axis], self.linearLimits.upperLimit[axis] = lo, hi
        else:
            self.angularLimits[axis - 3].loLimit, self.angularLimits[axis - 3].hiLimit = float(lo), float(hi)

    def setLinearLowerLimit(self, v):
        self.linearLimits.lowerLimit[:] = v

    def setLinearUpperLimit(self, v):
        self.linearLimits.upperLimit[:] = v

    def setAngularLowerLimit(self, v):
        for i in range(3):
            self.angularLimits[i].loLimit = float(v[i])

    def setAngularUpperLimit(self, v):
        for i in range(3):
            self.angularLimits[i].hiLimit = float(v[i])

    def getRotationalLimitMotor(self, index):
        return self.angularLimits[index]

    def getTranslationalLimitMotor(self):
        return self.linearLimits

    def getRigidBodyA(self):
        return self.rbA

    def getRigidBodyB(self):
        return self.rbB

    def getFrameOffsetA(self):
        return Transform(self.frameInA.basis.copy(), self.frameInA.origin.copy())

    def getFrameOffsetB(self):
        return Transform(self.frameInB.basis.copy(), self.frameInB.origin.copy())

    def _settings(self):
        L = self.linearLimits
        return (tuple(L.lowerLimit.tolist()), tuple(L.upperLimit.tolist()), L.limitSoftness, L.damping, L.restitution,
                tuple((m.loLimit, m.hiLimit, m.enableMotor, m.targetVelocity, m.maxMotorForce, m.maxLimitForce, m.damping,
                       m.limitSoftness, m.ERP, m.bounce) for m in self.angularLimits))

    def _push(self):
        g = self._world._g if self._world is not None else None
        if g is None or self._id is None:
            return
        st = self._settings()
        if st == self._sent:
            return
        L = self.linearLimits
        for i in range(3):
            g.set_6dof_limit(self._id, i, float(L.lowerLimit[i]), float(L.upperLimit[i]))
        g.set_6dof_linear_motor(self._id, L.limitSoftness, L.damping, L.restitution)
        for i, m in enumerate(self.angularLimits):
            g.set_6dof_limit(self._id, 3 + i, m.loLimit, m.hiLimit)
            g.set_6dof_angular_motor(self._id, i, m.enableMotor, m.targetVelocity, m.maxMotorForce, m.maxLimitForce,
                                     m.damping, m.limitSoftness, m.ERP, m.bounce)
        self._sent = st

    def getAppliedImpulse(self):
        return 0.0    # the reference's 6-dof joint leaves TypedConstraint.appliedImpulse at 0


class ClosestRayResultCallback:
    """CollisionWorld.ClosestRayResultCallback (collision/dispatch/CollisionWorld.java:697-729)."""

    def __init__(self, rayFromWorld, rayToWorld):
        self.rayFromWorld = np.asarray(rayFromWorld, np.float32).reshape(3).copy()
        self.rayToWorld = np.asarray(rayToWorld, np.float32).reshape(3).copy()
        self.closestHitFraction = 1.0
        self.collisionObject = None
        self.collisionFilterGroup = 1      # CollisionFilterGroups.DEFAULT_FILTER
        self.collisionFilterMask = -1      # CollisionFilterGroups.ALL_FILTER
        self.hitNormalWorld = np.zeros(3, np.float32)
        self.hitPointWorld = np.zeros(3, np.float32)

    def hasHit(self):
        return self.collisionObject is not None


class ClosestConvexResultCallback:
    """CollisionWorld.ClosestConvexResultCallback (collision/dispatch/CollisionWorld.java:794-836)."""

    def __init__(self, convexFromWorld, convexToWorld):
        self.convexFromWorld = np.asarray(convexFromWorld, np.float32).reshape(3).copy()
        self.convexToWorld = np.asarray(convexToWorld, np.float32).reshape(3).copy()
        self.closestHitFraction = 1.0
        self.hitCollisionObject = None
        self.collisionFilterGroup = 1
        self.collisionFilterMask = -1
        self.hitNormalWorld = np.zeros(3, np.float32)
        self.hitPointWorld = np.zeros(3, np.float32)

    def hasHit(self):
        return self.hitCollisionObject is not None


class DiscreteDynamicsWorld:
    def __init__(self, dispatcher=None, pairCache=None, constraintSolver=None, collisionConfiguration=None, device=0):
        self._gravity = (0.0, -10.0, 0.0)
        self._solver = ContactSolverInfo()
        self._device = device
        self._bodies = []
        self._shapes = []
        self._g = None
        self._forces = self._torques = None
        self._uploaded = 0
        self._constraints = []
        self._sent = 0
        self._tick_cb = None
        self._world_user_info = None

    # -- configuration (before the first step) --
    def setGravity(self, g):
        """DiscreteDynamicsWorld.setGravity: the world's gravity and RigidBody.setGravity of every body."""
        self._gravity = tuple(float(x) for x in g)
        if self._g is not None:
            self._g.set_gravity(self._gravity)
        for b in self._bodies:
            b._gravity_acc = None   # the world's call overrides a body's own setGravity staged before upload

    def getGravity(self):
        return self._gravity

    def getSolverInfo(self):
        return self._solver

    def addRigidBody(self, body, group=None, mask=None):
        if self._g is not None and self._uploaded != len(self._bodies):
            raise RuntimeError("internal: bodies not uploaded")
        body._world = self
        body._index = len(self._bodies)
        if group is not None:
            body._group, body._mask = int(group), int(mask)
        self._bodies.append(body)
        if self._g is not None:
            self._upload()

    def removeRigidBody(self, body):
        """DiscreteDynamicsWorld.removeRigidBody: the body leaves the world with its pairs and
        manifolds; the bodies after it move down (their _index drops by one)."""
        if body._world is not self:
            return
        i = body._index
        for c in self._constraints:
            if c.rbA is body or getattr(c, "rbB", None) is body:
                raise RuntimeError("removeRigidBody of a body a constraint uses (remove the constraint first)")
        if self._g is not None and i < self._uploaded:
            self._g.remove_bodies([i])
            self._uploaded -= 1
        del self._bodies[i]
        for b in self._bodies[i:]:
            b._index -= 1
        if self._forces is not None and i < len(self._forces):
            self._forces = np.delete(self._forces, i, 0)
            self._torques = np.delete(self._torques, i, 0)
        self._cache = None
        body._world = None
        body._index = None

    def getNumCollisionObjects(self):
        return len(self._bodies)

    def addConstraint(self, constraint, disableCollisionsBetweenLinkedBodies=False):
        """DiscreteDynamicsWorld.addConstraint (java:515-521).  Linked bodies keep colliding:
        disableCollisionsBetweenLinkedBodies = True is not supported."""
        if disableCollisionsBetweenLinkedBodies:
            raise NotImplementedError("disableCollisionsBetweenLinkedBodies is not supported by the GPU world")
        constraint._world = self
        self._constraints.append(constraint)

    def getNumConstraints(self):
        return len(self._constraints)

    def getConstraint(self, i):
        return self._constraints[i]

    def removeConstraint(self, constraint):
        """DiscreteDynamicsWorld.removeConstraint (java:524-528): the constraints after it move down."""
        if constraint not in self._constraints:
            return
        k = self._constraints.index(constraint)
        if constraint._id is not None:
            self._g.remove_joint(constraint._id)
            for c in self._constraints[k + 1:]:
                if c._id is not None:
                    c._id -= 1
            self._sent -= 1
        del self._constraints[k]
        constraint._id = None
        constraint._world = None

    def getCollisionObjectArray(self):
        return list(self._bodies)

    # DiscreteDynamicsWorld.clearForces / applyGravity (java:226-250): on the device accumulators
    def clearForces(self):
        self._forces = self._torques = None
        self._ensure().stage(_abi.STAGE_CLEAR_FORCES)
        self._cache = None

    def applyGravity(self):
        self._flush_forces()
        self._ensure().stage(_abi.STAGE_APPLY_GRAVITY)
        self._cache = None

    # DynamicsWorld.setInternalTickCallback (DynamicsWorld.java:141-144): cb.internalTick(world,
    # timeStep) (or cb(world, timeStep)) after every substep; forces it applies act from the next
    # substep on, as the reference's accumulators do
    def setInternalTickCallback(self, cb, worldUserInfo=None):
        self._tick_cb = cb
        self._world_user_info = worldUserInfo
        if self._g is not None:
            self._install_tick()

    def getWorldUserInfo(self):
        return self._world_user_info

    def setWorldUserInfo(self, info):
        self._world_user_info = info

    def _install_tick(self):
        cb = self._tick_cb
        if cb is None:
            self._g.set_internal_tick_callback(None)
            return
        fn = cb.internalTick if hasattr(cb, "internalTick") else cb

        def tick(_g, dt):
            self._cache = None
            fn(self, dt)
            self._flush_forces()
            self._cache = None
        self._g.set_internal_tick_callback(tick)

    # -- stepping --
    def _ensure(self):
        if self._g is None:
            s = self._solver
            cfg = _abi.default_config(gravity=self._gravity)
            cfg.num_iterations = s.numIterations
            cfg.erp = s.erp
            cfg.warmstarting_factor = s.warmstartingFactor
            cfg.linear_slop = s.linearSlop
            cfg.solver_mode = s.solverMode
            cfg.device = self._device
            self._g = GpuWorld(config=cfg)
            if self._tick_cb is not None:
                self._install_tick()
        if self._uploaded != len(self._bodies):
            self._upload()
        for c in self._constraints[self._sent:]:
            b = -1 if c.rbB is None else c.rbB._index
            if isinstance(c, HingeConstraint):
                c._id = self._g.add_hinge(c.rbA._index, b, c.frameA.as12(), c.frameB.as12())
                c._push()
                continue
            if isinstance(c, SliderConstraint):
                c._id = self._g.add_slider(c.rbA._index, b, c.frameInA.as12(), c.frameInB.as12(),
                                           c.useLinearReferenceFrameA)
                c._push()
                continue
            if isinstance(c, ConeTwistConstraint):
                c._id = self._g.add_cone_twist(c.rbA._index, b, c.frameA.as12(), c.frameB.as12())
                c._push()
                continue
            if isinstance(c, Generic6DofConstraint):
                c._id = self._g.add_generic6dof(c.rbA._index, b, c.frameInA.as12(), c.frameInB.as12(),
                                                c.useLinearReferenceFrameA)
                c._push()
                continue
            c._id = self._g.add_point2point(c.rbA._index, b, c.pivotInA, c.pivotInB)
            st = c.setting
            self._g.set_joint_setting(c._id, st.tau, st.damping, st.impulseClamp)
        self._sent = len(self._constraints)
        return self._g

    def _upload(self):
        from .scenes import BODY_DTYPE, Scene
        new = self._bodies[self._uploaded:]
        shapes, ids = [], {}
        for b in new:
            sh = b.info.collisionShape
            if sh._id is None:
                ids[id(sh)] = len(self._shapes) + len(shapes)
                shapes.append(sh)
        recs = np.zeros(len(new), BODY_DTYPE)
        for k, b in enumerate(new):
            i = b.info
            sh = i.collisionShape
            recs[k]["mass"] = i.mass
            recs[k]["shape"] = sh._id if sh._id is not None else ids[id(sh)]
            t = i.startWorldTransform
            if i.motionState is not None and hasattr(i.motionState, "getWorldTransform"):
                t = i.motionState.getWorldTransform()
            recs[k]["transform"] = t.as12()
            recs[k]["local_inertia"] = i.localInertia
            recs[k]["linear_damping"] = i.linearDamping
            recs[k]["angular_damping"] = i.angularDamping
            recs[k]["friction"] = i.friction
            recs[k]["restitution"] = i.restitution
            recs[k]["linear_sleeping_threshold"] = i.linearSleepingThreshold
            recs[k]["angular_sleeping_threshold"] = i.angularSleepingThreshold
            recs[k]["linear_velocity"] = b._linvel
            recs[k]["angular_velocity"] = b._angvel
            recs[k]["collision_group"] = b._group
            recs[k]["collision_flags"] = b._flags
            recs[k]["activation_state"] = b._activation
            recs[k]["collision_mask"] = b._mask
        sc = Scene("staged", 0, 0, {}, [s.desc() for s in shapes], recs)
        g = self._g
        if shapes:
            from . import lib
            descs = sc.shape_descs()
            lib.check(lib.lib().jbgpu_world_add_shapes(g.h, descs, len(descs), None))
            for s in shapes:
                s._id = ids[id(s)]
                s._world = self
        self._shapes += shapes
        b, ptr = sc.body_descs_ptr()
        from . import lib
        lib.check(lib.lib().jbgpu_world_add_bodies(g.h, ptr, len(b), None))
        self._uploaded = len(self._bodies)
        grav = [b for b in new if b._gravity_acc is not None]
        if grav:   # addRigidBody set the world's gravity; a later setGravity of the body overrides it
            g.set_body_gravity([b._index for b in grav], [b._gravity_acc for b in grav])
            for b in grav:
                b._gravity_acc = None
        ccd = [b for b in new if b._ccd != (0.0, 0.0)]
        if ccd:
            g.set_ccd([b._index for b in ccd], [b._ccd[0] for b in ccd], [b._ccd[1] for b in ccd])

    def _pending_force(self, index, force=None, torque=None):
        """Forces and torques applied since the last flush, summed per body in call order."""
        n = len(self._bodies)
        if self._forces is None:
            self._forces = np.zeros((n, 3), F32)
            self._torques = np.zeros((n, 3), F32)
        elif len(self._forces) < n:
            pad = np.zeros((n - len(self._forces), 3), F32)
            self._forces = np.concatenate([self._forces, pad])
            self._torques = np.concatenate([self._torques, pad])
        if force is not None:
            self._forces[index] += np.asarray(force, F32)
        if torque is not None:
            self._torques[index] += np.asarray(torque, F32)

    def _flush_forces(self):
        """The pending forces and torques added to the device accumulators."""
        if self._forces is None:
            return
        g = self._ensure()
        n = len(self._bodies)
        f, t = self._forces, self._torques
        if len(f) < n:
            pad = np.zeros((n - len(f), 3), F32)
            f, t = np.concatenate([f, pad]), np.concatenate([t, pad])
        self._forces = self._torques = None
        g.apply_forces(f, t if np.any(t) else None)
        self._cache = None

    def stepSimulation(self, timeStep, maxSubSteps=1, fixedTimeStep=1.0 / 60.0):
        g = self._ensure()
        for c in self._constraints:
            if isinstance(c, (Generic6DofConstraint, SliderConstraint)):
                c._push()
        self._flush_forces()
        # saveKinematicState reads a kinematic body's motion state (RigidBody.java:190-205): its
        # pose is written to the world first, for the bodies that are not ISLAND_SLEEPING
        kin = [b for b in self._bodies if b.isKinematicObject() and b.info.motionState is not None and
               hasattr(b.info.motionState, "getWorldTransform")]
        if kin:
            st = self._state()
            t = st["transform"].copy()
            for b in kin:
                if st["activation_state"][b._index] != ISLAND_SLEEPING:
                    t[b._index] = b.info.motionState.getWorldTransform().as12()
            g.set_state({"transform": t})
            self._cache = None
        n = g.step_simulation(timeStep, maxSubSteps, fixedTimeStep)
        self._cache = None
        self._synchronize_motion_states(g)
        return n

    def _synchronize_motion_states(self, g):
        """synchronizeMotionStates (java:251-276): MotionState.setWorldTransform of every dynamic
        body that has one, with the interpolated transform (once per stepSimulation call: the
        reference's calls after each substep hand over the same values for the last one)."""
        dyn = [b for b in self._bodies if b.info.motionState is not None and not b.isStaticOrKinematicObject()
               and hasattr(b.info.motionState, "setWorldTransform")]
        if not dyn:
            return
        xf = g.get_interpolated_transforms()
        for b in dyn:
            b.info.motionState.setWorldTransform(Transform.from12(xf[b._index]))

    # -- queries --
    def rayTest(self, rayFromWorld, rayToWorld, resultCallback):
        """CollisionWorld.rayTest (collision/dispatch/CollisionWorld.java:553-591) with a
        ClosestRayResultCallback, on the GPU world's bodies as the last step left them."""
        cb = resultCallback
        h = self._ensure().ray_test([rayFromWorld], [rayToWorld], group=cb.collisionFilterGroup,
                                    mask=cb.collisionFilterMask)[0]
        if h["body"] >= 0:
            cb.closestHitFraction = float(h["fraction"])
            cb.collisionObject = self._bodies[int(h["body"])]
            cb.hitNormalWorld = h["normal"].copy()
            cb.hitPointWorld = h["point"].copy()

    def convexSweepTest(self, castShape, convexFromWorld, convexToWorld, resultCallback):
        """CollisionWorld.convexSweepTest (collision/dispatch/CollisionWorld.java:596-645) with a
        ClosestConvexResultCallback; from / to are Transforms.  Raises RuntimeError where the
        reference throws: when the sweep's path reaches a static plane."""
        g = self._ensure()
        if castShape._id is None:
            from .scenes import Scene
            from . import lib
            descs = Scene("cast", 0, 0, {}, [castShape.desc()], np.zeros(0)).shape_descs()
            lib.check(lib.lib().jbgpu_world_add_shapes(g.h, descs, 1, None))
            castShape._id = len(self._shapes)
            self._shapes.append(castShape)
        cb = resultCallback
        h = g.convex_sweep_test(castShape._id, [convexFromWorld.as12()], [convexToWorld.as12()],
                                group=cb.collisionFilterGroup, mask=cb.collisionFilterMask)[0]
        if h["body"] == -2:
            raise RuntimeError("convexSweepTest reached a static plane (the reference throws there)")
        if h["body"] >= 0:
            cb.closestHitFraction = float(h["fraction"])
            cb.hitCollisionObject = self._bodies[int(h["body"])]
            cb.hitNormalWorld = h["normal"].copy()
            cb.hitPointWorld = h["point"].copy()

    # -- state access --
    _cache = None

    def _state(self):
        if self._cache is None:
            self._cache = self._ensure().get_state()
        return self._cache

    def _get_field(self, field, index):
        return self._state()[field][index].copy()

    def _set_field(self, field, index, value):
        st = self._state()
        st[field][index] = value
        self._g.set_state({field: st[field]})
        self._cache = None

    def getDispatcher(self):
        return _Dispatcher(self)

    # CollisionWorld.updateAabbs / performDiscreteCollisionDetection (collision/dispatch/
    # CollisionWorld.java:101-155): the collision half of a step without the dynamics, e.g. to
    # read contacts after moving bodies by hand
    def updateAabbs(self):
        self._ensure().stage(_abi.STAGE_AABB)
        self._cache = None

    def performDiscreteCollisionDetection(self):
        g = self._ensure()
        for st in (_abi.STAGE_AABB, _abi.STAGE_PAIRS, _abi.STAGE_NARROWPHASE):
            g.stage(st)
        self._cache = None

    def getWorldType(self):
        return "DISCRETE_DYNAMICS_WORLD"   # DynamicsWorldType

    def getConstraintSolver(self):
        return self._solver

    def setNumTasks(self, n):
        """DiscreteDynamicsWorld.setNumTasks is a no-op in the reference too (java:1084-1085)."""

    def getPairCache(self):
        return self._ensure().get_pairs()

    def close(self):
        if self._g is not None:
            self._g.close()
            self._g = None


class _Dispatcher:
    """CollisionDispatcher read access: getNumManifolds / getManifoldByIndexInternal."""

    def __init__(self, world):
        self._m = world._ensure().get_manifolds()

    def getNumManifolds(self):
        return int(np.sum(self._m["flags"] & 1))

    def getManifoldByIndexInternal(self, i):
        idx = np.nonzero(self._m["flags"] & 1)[0][i]
        return {"key": int(self._m["keys"][idx]), "numContacts": int(self._m["num_points"][idx]),
                "points": self._m["points"][idx, :self._m["num_points"][idx]]}
