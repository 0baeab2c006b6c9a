"""HingeConstraint's constraint frames, computed as the reference's constructors compute them.

A hinge is uploaded with its two frames (rbAFrame, rbBFrame: 3x3 basis row-major, then the
origin; z is the hinge axis), the state HingeConstraint holds after construction
(dynamics/constraintsolver/HingeConstraint.java:82-236).  A Java caller reads them from its
HingeConstraint object; these functions give the same frames to Python callers, in binary32
with the reference's operation order: QuaternionUtil.shortestArcQuat / quatRotate
(linearmath/QuaternionUtil.java:49-90) and libGDX Vector3/Quaternion arithmetic.
"""
import math

import numpy as np

F = np.float32
FLT_EPSILON = F(1.19209290e-07)


def _v(a):
    return [F(x) for x in np.asarray(a, np.float32).reshape(3)]


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _crs(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _col(m, c):
    return [F(m[0][c]), F(m[1][c]), F(m[2][c])]


def _mulMv(m, v):        # libGDX Vector3.mul(Matrix3): M * v
    return [F(m[r][0]) * v[0] + F(m[r][1]) * v[1] + F(m[r][2]) * v[2] for r in range(3)]


def shortest_arc_quat(v0, v1):
    """QuaternionUtil.shortestArcQuat: (x, y, z, w)."""
    c = _crs(v0, v1)
    d = _dot(v0, v1)
    if float(d) < -1.0 + float(FLT_EPSILON):          # compared in double, as the reference does
        return [F(0.0), F(1.0), F(0.0), F(0.0)]
    s = F(math.sqrt(float((F(1.0) + d) * F(2.0))))
    rs = F(1.0) / s
    return [c[0] * rs, c[1] * rs, c[2] * rs, s * F(0.5)]


def quat_rotate(q, v):
    """QuaternionUtil.quatRotate: q * v * q^-1 through QuaternionUtil.mul and Quaternion.mul."""
    x, y, z, w = q
    rx = w * v[0] + y * v[2] - z * v[1]
    ry = w * v[1] + z * v[0] - x * v[2]
    rz = w * v[2] + x * v[1] - y * v[0]
    rw = -x * v[0] - y * v[1] - z * v[2]
    ox, oy, oz, ow = -x, -y, -z, w
    nx = rw * ox + rx * ow + ry * oz - rz * oy
    ny = rw * oy + ry * ow + rz * ox - rx * oz
    nz = rw * oz + rz * ow + rx * oy - ry * ox
    return [nx, ny, nz]


def _frame(c0, c1, c2, origin):
    """Frame with the given basis columns: MatrixUtil.setRow(basis, r, c0[r], c1[r], c2[r])."""
    out = np.zeros(12, np.float32)
    for r in range(3):
        out[r * 3:r * 3 + 3] = (c0[r], c1[r], c2[r])
    out[9:] = origin
    return out


def hinge_frames_two_bodies(basis_a, pivot_in_a, pivot_in_b, axis_in_a, axis_in_b):
    """HingeConstraint(rbA, rbB, pivotInA, pivotInB, axisInA, axisInB) (java:82-131).
    basis_a: rbA's centre-of-mass basis (3x3, row-major).  Returns (frame_a, frame_b)."""
    m = np.asarray(basis_a, np.float32).reshape(3, 3)
    axa, axb = _v(axis_in_a), _v(axis_in_b)
    a1 = _col(m, 0)
    projection = _dot(axa, a1)
    if projection >= F(1.0) - FLT_EPSILON:
        a1 = [x * F(-1) for x in _col(m, 2)]
        a2 = _col(m, 1)
    elif projection <= F(-1.0) + FLT_EPSILON:
        a1 = _col(m, 2)
        a2 = _col(m, 1)
    else:
        a2 = _crs(axa, a1)
        a1 = _crs(a2, axa)
    frame_a = _frame(a1, a2, axa, _v(pivot_in_a))
    arc = shortest_arc_quat(axa, axb)
    b1 = quat_rotate(arc, a1)
    b2 = _crs(axb, b1)
    frame_b = _frame(b1, b2, [-x for x in axb], _v(pivot_in_b))
    return frame_a, frame_b


def hinge_frames_one_body(transform_a, pivot_in_a, axis_in_a):
    """HingeConstraint(rbA, pivotInA, axisInA) (java:133-184): body B is the fixed body and its
    frame sits at the pivot's current world position.  transform_a: rbA's centre-of-mass
    transform (12 floats: basis row-major, origin)."""
    t = np.asarray(transform_a, np.float32).reshape(12)
    m = t[:9].reshape(3, 3)
    axa = _v(axis_in_a)
    a1 = _col(m, 0)
    projection = _dot(a1, axa)
    if projection > FLT_EPSILON:
        a1 = [a1[i] * projection for i in range(3)]
        a1 = [a1[i] - axa[i] for i in range(3)]
    else:
        a1 = _col(m, 1)
    a2 = _crs(axa, a1)
    pa = _v(pivot_in_a)
    frame_a = _frame(a1, a2, axa, pa)
    axb = _mulMv(m, [x * F(-1) for x in axa])
    arc = shortest_arc_quat(axa, axb)
    b1 = quat_rotate(arc, a1)
    b2 = _crs(axb, b1)
    origin = [p + F(o) for p, o in zip(_mulMv(m, pa), t[9:])]   # Transform.transform
    frame_b = _frame(b1, b2, axb, origin)
    return frame_a, frame_b


def hinge_frames_from_frames(transform_a, frame_a, frame_b=None):
    """HingeConstraint(rbA, rbB, rbAFrame, rbBFrame) (java:186-210) and HingeConstraint(rbA,
    rbAFrame) (java:212-236): B's frame has its z column negated; without rbBFrame it is
    rbAFrame at the pivot's current world position."""
    fa = np.asarray(frame_a, np.float32).reshape(12).copy()
    if frame_b is not None:
        fb = np.asarray(frame_b, np.float32).reshape(12).copy()
    else:
        fb = fa.copy()
        t = np.asarray(transform_a, np.float32).reshape(12)
        o = _mulMv(t[:9].reshape(3, 3), _v(fa[9:]))
        fb[9:] = [o[i] + F(t[9 + i]) for i in range(3)]
    for r in range(3):
        fb[r * 3 + 2] = fb[r * 3 + 2] * F(-1)
    return fa, fb
