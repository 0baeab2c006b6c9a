// ORACLE (test infrastructure only): CPU restatement of the reference's FP32 arithmetic.
// Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
//
// Java float semantics: every operation is an IEEE-754 binary32 operation evaluated left
// to right with no contraction (build with -ffp-contract=off); Math.sqrt/sin/cos/pow/acos
// evaluate in binary64 and the result is rounded to float by the cast.
//
// libGDX math (com.badlogic.gdx.math.Vector3 / Matrix3 / Quaternion) is a third-party
// dependency that the reference does not vendor and does not pin (no build file;
// src/BulletPhysics.gwt.xml:4 inherits com.badlogic.gdx).  The routines below restate its
// published behaviour (libGDX 1.x): Vector3.nor() skips when len2 is exactly 0 or 1,
// Quaternion.nor() skips when |len2 - 1| <= 1e-6, Vector3.mul(Matrix3) computes M*v,
// Matrix3.mul(B) computes this*B, Quaternion.setFromMatrix(true, m) normalises the rows
// and uses the trace/largest-diagonal branches with the "1.0 + ..." sums in double.
// No reference test pins results at this boundary: parity there is unpinned.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace jb {

static inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// Java Float.floatToIntBits equality (all NaNs collapse to one pattern), used by
// libGDX Vector3.equals.
static inline bool java_feq_bits(float a, float b) {
    if (a != a && b != b) return true;
    return fbits(a) == fbits(b);
}
// java.lang.Math.max(float,float) / min(float,float)
static inline float jmax(float a, float b) {
    if (a != a) return a;
    if (a == 0.0f && b == 0.0f && (fbits(a) & 0x80000000u)) return b;
    return (a >= b) ? a : b;
}
static inline float jmin(float a, float b) {
    if (a != a) return a;
    if (a == 0.0f && b == 0.0f) return (fbits(b) & 0x80000000u) ? b : a;
    return (a <= b) ? a : b;
}
static inline float jsqrt(float x) { return (float)std::sqrt((double)x); }
static inline float jsin(float x) { return (float)std::sin((double)x); }
static inline float jcos(float x) { return (float)std::cos((double)x); }
static inline float jacos(float x) { return (float)std::acos((double)x); }
static inline float jpow(float a, float b) { return (float)std::pow((double)a, (double)b); }

static const float FLT_EPS = 1.19209290e-07f;           // BulletGlobals.FLT_EPSILON
static const float SIMD_2_PI = 6.283185307179586232f;     // BulletGlobals.java:42
static const float SIMD_PI = SIMD_2_PI * 0.5f;
static const float SIMD_HALF_PI = SIMD_2_PI * 0.25f;
static const float SIMD_INFINITY = 3.40282347e+38f;       // Float.MAX_VALUE

struct V3 { float x, y, z; };
static inline V3 v3(float x, float y, float z) { V3 r = {x, y, z}; return r; }
static inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 scl(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 mulc(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }  // VectorUtil.mul / Vector3.scl(Vector3)
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 crs(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float len2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline float len(V3 a) { return jsqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline V3 nor(V3 a) {   // libGDX Vector3.nor()
    float l2 = len2(a);
    if (l2 == 0.0f || l2 == 1.0f) return a;
    return scl(a, 1.0f / jsqrt(l2));
}
static inline bool v3_equals(V3 a, V3 b) { return java_feq_bits(a.x, b.x) && java_feq_bits(a.y, b.y) && java_feq_bits(a.z, b.z); }
static inline float coord(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
static inline void set_coord(V3& v, int i, float f) { if (i == 0) v.x = f; else if (i == 1) v.y = f; else v.z = f; }

// Matrix3, stored row-major m[r][c] (libGDX stores column-major; only the maths matters).
struct M3 { float m[3][3]; };
static inline M3 m3_identity() { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = (i == j) ? 1.0f : 0.0f; return r; }
// Vector3.mul(Matrix3): M * v
static inline V3 mulMv(V3 v, const M3& M) {
    return v3(v.x * M.m[0][0] + v.y * M.m[0][1] + v.z * M.m[0][2],
              v.x * M.m[1][0] + v.y * M.m[1][1] + v.z * M.m[1][2],
              v.x * M.m[2][0] + v.y * M.m[2][1] + v.z * M.m[2][2]);
}
// MatrixUtil.transposeTransform: M^T * v (linearmath/MatrixUtil.java:265-285)
static inline V3 mulMTv(V3 v, const M3& M) {
    return v3(M.m[0][0] * v.x + M.m[1][0] * v.y + M.m[2][0] * v.z,
              M.m[0][1] * v.x + M.m[1][1] * v.y + M.m[2][1] * v.z,
              M.m[0][2] * v.x + M.m[1][2] * v.y + M.m[2][2] * v.z);
}
// Matrix3.mul(B): this * B
static inline M3 mulMM(const M3& A, const M3& B) {
    M3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            r.m[i][j] = A.m[i][0] * B.m[0][j] + A.m[i][1] * B.m[1][j] + A.m[i][2] * B.m[2][j];
    return r;
}
static inline M3 transpose(const M3& A) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[j][i]; return r; }
static inline M3 absM(const M3& A) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = std::fabs(A.m[i][j]); return r; }
// MatrixUtil.scale: dest[r][c] = mat[r][c] * s[c] (linearmath/MatrixUtil.java:205-215)
static inline M3 scaleM(const M3& A, V3 s) {
    M3 r;
    for (int i = 0; i < 3; i++) { r.m[i][0] = A.m[i][0] * s.x; r.m[i][1] = A.m[i][1] * s.y; r.m[i][2] = A.m[i][2] * s.z; }
    return r;
}
static inline V3 row(const M3& A, int i) { return v3(A.m[i][0], A.m[i][1], A.m[i][2]); }

struct Quat { float x, y, z, w; };
static inline Quat quat(float x, float y, float z, float w) { Quat q = {x, y, z, w}; return q; }
// libGDX Quaternion.mul(other): this * other
static inline Quat qmul(Quat a, Quat o) {
    float nx = a.w * o.x + a.x * o.w + a.y * o.z - a.z * o.y;
    float ny = a.w * o.y + a.y * o.w + a.z * o.x - a.x * o.z;
    float nz = a.w * o.z + a.z * o.w + a.x * o.y - a.y * o.x;
    float nw = a.w * o.w - a.x * o.x - a.y * o.y - a.z * o.z;
    return quat(nx, ny, nz, nw);
}
// libGDX Quaternion.nor()
static inline Quat qnor(Quat q) {
    float l = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (l != 0.0f && !(std::fabs(l - 1.0f) <= 0.000001f)) {
        l = jsqrt(l);
        q.w = q.w / l; q.x = q.x / l; q.y = q.y / l; q.z = q.z / l;
    }
    return q;
}
// libGDX Quaternion.setFromMatrix(true, m) -> setFromAxes(true, m00, m01, m02, m10, ..., m22)
static inline Quat q_from_matrix(const M3& M) {
    float xx = M.m[0][0], xy = M.m[0][1], xz = M.m[0][2];
    float yx = M.m[1][0], yy = M.m[1][1], yz = M.m[1][2];
    float zx = M.m[2][0], zy = M.m[2][1], zz = M.m[2][2];
    {
        const float lx = 1.0f / jsqrt(xx * xx + xy * xy + xz * xz);
        const float ly = 1.0f / jsqrt(yx * yx + yy * yy + yz * yz);
        const float lz = 1.0f / jsqrt(zx * zx + zy * zy + zz * zz);
        xx *= lx; xy *= lx; xz *= lx;
        yx *= ly; yy *= ly; yz *= ly;
        zx *= lz; zy *= lz; zz *= lz;
    }
    const float t = xx + yy + zz;
    Quat q;
    if (t >= 0) {
        float s = jsqrt(t + 1);
        q.w = 0.5f * s;
        s = 0.5f / s;
        q.x = (zy - yz) * s;
        q.y = (xz - zx) * s;
        q.z = (yx - xy) * s;
    } else if ((xx > yy) && (xx > zz)) {
        float s = (float)std::sqrt(1.0 + (double)xx - (double)yy - (double)zz);
        q.x = s * 0.5f;
        s = 0.5f / s;
        q.y = (yx + xy) * s;
        q.z = (xz + zx) * s;
        q.w = (zy - yz) * s;
    } else if (yy > zz) {
        float s = (float)std::sqrt(1.0 + (double)yy - (double)xx - (double)zz);
        q.y = s * 0.5f;
        s = 0.5f / s;
        q.x = (yx + xy) * s;
        q.z = (zy + yz) * s;
        q.w = (xz - zx) * s;
    } else {
        float s = (float)std::sqrt(1.0 + (double)zz - (double)xx - (double)yy);
        q.z = s * 0.5f;
        s = 0.5f / s;
        q.x = (xz + zx) * s;
        q.y = (zy + yz) * s;
        q.w = (yx - xy) * s;
    }
    return q;
}
// MatrixUtil.setRotation (linearmath/MatrixUtil.java:287-304)
static inline M3 m3_from_quat(Quat q) {
    float d = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    float s = 2.0f / d;
    float xs = q.x * s, ys = q.y * s, zs = q.z * s;
    float wx = q.w * xs, wy = q.w * ys, wz = q.w * zs;
    float xx = q.x * xs, xy = q.x * ys, xz = q.x * zs;
    float yy = q.y * ys, yz = q.y * zs, zz = q.z * zs;
    M3 r;
    r.m[0][0] = 1.0f - (yy + zz); r.m[0][1] = xy - wz;          r.m[0][2] = xz + wy;
    r.m[1][0] = xy + wz;          r.m[1][1] = 1.0f - (xx + zz); r.m[1][2] = yz - wx;
    r.m[2][0] = xz - wy;          r.m[2][1] = yz + wx;          r.m[2][2] = 1.0f - (xx + yy);
    return r;
}
// QuaternionUtil.setRotation(q, axis, angle) (linearmath/QuaternionUtil.java:41-46)
static inline Quat q_axis_angle(V3 axis, float angle) {
    float d = len(axis);
    float s = jsin(angle * 0.5f) / d;
    return quat(axis.x * s, axis.y * s, axis.z * s, jcos(angle * 0.5f));
}

// Transform (linearmath/Transform.java)
struct Xf { M3 b; V3 o; };
static inline Xf xf_identity() { Xf t; t.b = m3_identity(); t.o = v3(0, 0, 0); return t; }
static inline V3 xf_apply(const Xf& t, V3 v) { return add(mulMv(v, t.b), t.o); }           // transform(v)
static inline Xf xf_inverse(Xf t) { t.b = transpose(t.b); t.o = scl(t.o, -1.0f); t.o = mulMv(t.o, t.b); return t; }
static inline Xf xf_mul(const Xf& a, const Xf& b) { Xf r; r.o = xf_apply(a, b.o); r.b = mulMM(a.b, b.b); return r; }
static inline V3 xf_invXform(const Xf& t, V3 in) { V3 out = sub(in, t.o); return mulMv(out, transpose(t.b)); }

// MatrixUtil.invert (linearmath/MatrixUtil.java:362-395): cofactors over the determinant.
static inline M3 m3_invert(const M3& m) {
    auto cofac = [&](int r1, int c1, int r2, int c2) { return m.m[r1][c1] * m.m[r2][c2] - m.m[r1][c2] * m.m[r2][c1]; };
    float co_x = cofac(1, 1, 2, 2), co_y = cofac(1, 2, 2, 0), co_z = cofac(1, 0, 2, 1);
    float det = m.m[0][0] * co_x + m.m[0][1] * co_y + m.m[0][2] * co_z;
    float s = 1.0f / det;
    M3 r;
    r.m[0][0] = co_x * s;
    r.m[0][1] = cofac(0, 2, 2, 1) * s;
    r.m[0][2] = cofac(0, 1, 1, 2) * s;
    r.m[1][0] = co_y * s;
    r.m[1][1] = cofac(0, 0, 2, 2) * s;
    r.m[1][2] = cofac(0, 2, 1, 0) * s;
    r.m[2][0] = co_z * s;
    r.m[2][1] = cofac(0, 1, 2, 0) * s;
    r.m[2][2] = cofac(0, 0, 1, 1) * s;
    return r;
}

// TransformUtil.planeSpace1 (linearmath/TransformUtil.java:45-61)
static const float SIMDSQRT12 = 0.7071067811865475244008443621048490f;
static inline void plane_space1(V3 n, V3& p, V3& q) {
    if (std::fabs(n.z) > SIMDSQRT12) {
        float a = n.y * n.y + n.z * n.z;
        float k = 1.0f / jsqrt(a);
        p = v3(0, -n.z * k, n.y * k);
        q = v3(a * k, -n.x * p.z, n.x * p.y);
    } else {
        float a = n.x * n.x + n.y * n.y;
        float k = 1.0f / jsqrt(a);
        p = v3(-n.y * k, n.x * k, 0);
        q = v3(-n.z * p.y, n.z * p.x, a * k);
    }
}

// TransformUtil.integrateTransform (linearmath/TransformUtil.java:64-103)
static const float ANGULAR_MOTION_THRESHOLD = 0.5f * SIMD_HALF_PI;
static inline Xf integrate_transform(const Xf& cur, V3 linvel, V3 angvel, float dt) {
    Xf p;
    p.o.x = cur.o.x + dt * linvel.x;
    p.o.y = cur.o.y + dt * linvel.y;
    p.o.z = cur.o.z + dt * linvel.z;
    float fAngle = len(angvel);
    if (fAngle * dt > ANGULAR_MOTION_THRESHOLD) fAngle = ANGULAR_MOTION_THRESHOLD / dt;
    V3 axis;
    if (fAngle < 0.001f) {
        axis = scl(angvel, 0.5f * dt - (dt * dt * dt) * (0.020833333333f) * fAngle * fAngle);
    } else {
        axis = scl(angvel, jsin(0.5f * fAngle * dt) / fAngle);
    }
    Quat dorn = quat(axis.x, axis.y, axis.z, jcos(fAngle * dt * 0.5f));
    Quat orn0 = q_from_matrix(cur.b);
    Quat pred = qnor(qmul(dorn, orn0));
    p.b = m3_from_quat(pred);
    return p;
}

}  // namespace jb
