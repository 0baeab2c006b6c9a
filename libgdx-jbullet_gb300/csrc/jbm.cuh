// Device arithmetic with Java float semantics (the reference is Java: every float operation
// is IEEE binary32, evaluated left to right, never contracted; Math.sqrt/sin/cos/pow/acos are
// evaluated in binary64 and rounded by the float cast).  Translation units that include this
// header are compiled with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false.
//
// The libGDX math routines the reference calls (Vector3.nor/len/crs/dot, Matrix3.mul,
// Quaternion.mul/nor/setFromMatrix) are restated with libGDX 1.x semantics; see the
// matching functions below (linearmath/Transform.java:91-94, linearmath/MatrixUtil.java:287-362,
// linearmath/TransformUtil.java:64-103 of the reference).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define JBD __device__ __forceinline__
#define JBHD __host__ __device__ __forceinline__

namespace jbd {

struct V { float x, y, z; };
JBHD V mk(float x, float y, float z) { V r; r.x = x; r.y = y; r.z = z; return r; }
JBD V mk4(float4 a) { return mk(a.x, a.y, a.z); }
JBD float4 f4(V a, float w) { return make_float4(a.x, a.y, a.z, w); }
JBD V add(V a, V b) { return mk(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
JBD V sub(V a, V b) { return mk(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
JBD V scl(V a, float s) { return mk(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
JBD V mulc(V a, V b) { return mk(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)); }
JBD float dot(V a, V b) { return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z)); }
JBD V crs(V a, V b) {
    return mk(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
              __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
JBD float len2(V a) { return dot(a, a); }
JBD float jsqrt(float x) { return __fsqrt_rn(x); }     // == (float)Math.sqrt((double)x)
JBD float len(V a) { return jsqrt(len2(a)); }
JBD float jdiv(float a, float b) { return __fdiv_rn(a, b); }
JBD V nor(V a) {                                       // libGDX Vector3.nor()
    float l2 = len2(a);
    if (l2 == 0.0f || l2 == 1.0f) return a;
    return scl(a, jdiv(1.0f, jsqrt(l2)));
}
JBD float coord(V v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
JBD void set_coord(V& v, int i, float f) { if (i == 0) v.x = f; else if (i == 1) v.y = f; else v.z = f; }
JBD bool feq_bits(float a, float b) {                  // Float.floatToIntBits equality
    if (a != a && b != b) return true;
    return __float_as_uint(a) == __float_as_uint(b);
}
JBD bool vequals(V a, V b) { return feq_bits(a.x, b.x) && feq_bits(a.y, b.y) && feq_bits(a.z, b.z); }
JBD float jmax(float a, float b) {                     // java.lang.Math.max(float,float)
    if (a != a) return a;
    if (a == 0.0f && b == 0.0f && (__float_as_uint(a) & 0x80000000u)) return b;
    return (a >= b) ? a : b;
}
JBD float jmin(float a, float b) {                     // java.lang.Math.min(float,float)
    if (a != a) return a;
    if (a == 0.0f && b == 0.0f) return (__float_as_uint(b) & 0x80000000u) ? b : a;
    return (a <= b) ? a : b;
}
JBD float jsin(float x) { return (float)sin((double)x); }
JBD float jcos(float x) { return (float)cos((double)x); }
JBD float jpow(float a, float b) { return (float)pow((double)a, (double)b); }

constexpr float FLT_EPS = 1.19209290e-07f;
constexpr float SIMD_INFINITY = 3.40282347e+38f;
constexpr float SIMD_2_PI = 6.283185307179586232f;

// Row-major 3x3: r[i] is row i.
struct M { V r[3]; };
JBD V mulMv(V v, const M& m) {    // libGDX Vector3.mul(Matrix3): M * v
    return mk(dot(v, m.r[0]), dot(v, m.r[1]), dot(v, m.r[2]));
}
JBD V mulMTv(V v, const M& m) {   // MatrixUtil.transposeTransform: M^T * v
    return mk(__fadd_rn(__fadd_rn(__fmul_rn(m.r[0].x, v.x), __fmul_rn(m.r[1].x, v.y)), __fmul_rn(m.r[2].x, v.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m.r[0].y, v.x), __fmul_rn(m.r[1].y, v.y)), __fmul_rn(m.r[2].y, v.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m.r[0].z, v.x), __fmul_rn(m.r[1].z, v.y)), __fmul_rn(m.r[2].z, v.z)));
}
JBD M transpose(const M& a) {
    M t;
    t.r[0] = mk(a.r[0].x, a.r[1].x, a.r[2].x);
    t.r[1] = mk(a.r[0].y, a.r[1].y, a.r[2].y);
    t.r[2] = mk(a.r[0].z, a.r[1].z, a.r[2].z);
    return t;
}
JBD M mulMM(const M& a, const M& b) {   // libGDX Matrix3.mul: a * b
    M bt = transpose(b);
    M r;
    for (int i = 0; i < 3; i++) r.r[i] = mk(dot(a.r[i], bt.r[0]), dot(a.r[i], bt.r[1]), dot(a.r[i], bt.r[2]));
    return r;
}
JBD M absM(const M& a) {
    M r;
    for (int i = 0; i < 3; i++) r.r[i] = mk(fabsf(a.r[i].x), fabsf(a.r[i].y), fabsf(a.r[i].z));
    return r;
}
JBD M scaleM(const M& a, V s) {         // MatrixUtil.scale: column c scaled by s[c]
    M r;
    for (int i = 0; i < 3; i++) r.r[i] = mulc(a.r[i], s);
    return r;
}

struct Xf { M b; V o; };
JBD V xf_apply(const Xf& t, V v) { return add(mulMv(v, t.b), t.o); }
JBD Xf xf_inverse(Xf t) { t.b = transpose(t.b); t.o = scl(t.o, -1.0f); t.o = mulMv(t.o, t.b); return t; }
JBD Xf xf_mul(const Xf& a, const Xf& b) { Xf r; r.o = xf_apply(a, b.o); r.b = mulMM(a.b, b.b); return r; }
JBD V xf_invXform(const Xf& t, V in) { return mulMv(sub(in, t.o), transpose(t.b)); }

struct Q { float x, y, z, w; };
// MatrixUtil.invert (linearmath/MatrixUtil.java:362-395)
JBD M m3_invert(const M& m) {
    auto el = [&](int r, int c) { return coord(m.r[r], c); };
    auto cofac = [&](int r1, int c1, int r2, int c2) {
        return __fsub_rn(__fmul_rn(el(r1, c1), el(r2, c2)), __fmul_rn(el(r1, c2), el(r2, c1)));
    };
    const float co_x = cofac(1, 1, 2, 2), co_y = cofac(1, 2, 2, 0), co_z = cofac(1, 0, 2, 1);
    const float det = __fadd_rn(__fadd_rn(__fmul_rn(el(0, 0), co_x), __fmul_rn(el(0, 1), co_y)), __fmul_rn(el(0, 2), co_z));
    const float s = jdiv(1.0f, det);
    M r;
    r.r[0] = mk(__fmul_rn(co_x, s), __fmul_rn(cofac(0, 2, 2, 1), s), __fmul_rn(cofac(0, 1, 1, 2), s));
    r.r[1] = mk(__fmul_rn(co_y, s), __fmul_rn(cofac(0, 0, 2, 2), s), __fmul_rn(cofac(0, 2, 1, 0), s));
    r.r[2] = mk(__fmul_rn(co_z, s), __fmul_rn(cofac(0, 1, 2, 0), s), __fmul_rn(cofac(0, 0, 1, 1), s));
    return r;
}

JBD Q qmul(Q a, Q o) {                  // libGDX Quaternion.mul: a * o
    Q r;
    r.x = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.w, o.x), __fmul_rn(a.x, o.w)), __fmul_rn(a.y, o.z)), __fmul_rn(a.z, o.y));
    r.y = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.w, o.y), __fmul_rn(a.y, o.w)), __fmul_rn(a.z, o.x)), __fmul_rn(a.x, o.z));
    r.z = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.w, o.z), __fmul_rn(a.z, o.w)), __fmul_rn(a.x, o.y)), __fmul_rn(a.y, o.x));
    r.w = __fsub_rn(__fsub_rn(__fsub_rn(__fmul_rn(a.w, o.w), __fmul_rn(a.x, o.x)), __fmul_rn(a.y, o.y)), __fmul_rn(a.z, o.z));
    return r;
}
JBD Q qnor(Q q) {                       // libGDX Quaternion.nor: skipped when |len2-1| <= 1e-6
    float l = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(q.x, q.x), __fmul_rn(q.y, q.y)), __fmul_rn(q.z, q.z)), __fmul_rn(q.w, q.w));
    if (l != 0.0f && !(fabsf(__fsub_rn(l, 1.0f)) <= 0.000001f)) {
        l = jsqrt(l);
        q.w = jdiv(q.w, l); q.x = jdiv(q.x, l); q.y = jdiv(q.y, l); q.z = jdiv(q.z, l);
    }
    return q;
}
JBD Q q_from_matrix(const M& m) {       // libGDX Quaternion.setFromMatrix(true, m)
    float xx = m.r[0].x, xy = m.r[0].y, xz = m.r[0].z;
    float yx = m.r[1].x, yy = m.r[1].y, yz = m.r[1].z;
    float zx = m.r[2].x, zy = m.r[2].y, zz = m.r[2].z;
    const float lx = jdiv(1.0f, len(mk(xx, xy, xz)));
    const float ly = jdiv(1.0f, len(mk(yx, yy, yz)));
    const float lz = jdiv(1.0f, len(mk(zx, zy, zz)));
    xx = __fmul_rn(xx, lx); xy = __fmul_rn(xy, lx); xz = __fmul_rn(xz, lx);
    yx = __fmul_rn(yx, ly); yy = __fmul_rn(yy, ly); yz = __fmul_rn(yz, ly);
    zx = __fmul_rn(zx, lz); zy = __fmul_rn(zy, lz); zz = __fmul_rn(zz, lz);
    const float t = __fadd_rn(__fadd_rn(xx, yy), zz);
    Q q;
    if (t >= 0) {
        float s = jsqrt(__fadd_rn(t, 1.0f));
        q.w = __fmul_rn(0.5f, s);
        s = jdiv(0.5f, s);
        q.x = __fmul_rn(__fsub_rn(zy, yz), s);
        q.y = __fmul_rn(__fsub_rn(xz, zx), s);
        q.z = __fmul_rn(__fsub_rn(yx, xy), s);
    } else if ((xx > yy) && (xx > zz)) {
        float s = (float)__dsqrt_rn(__dsub_rn(__dsub_rn(__dadd_rn(1.0, (double)xx), (double)yy), (double)zz));
        q.x = __fmul_rn(s, 0.5f);
        s = jdiv(0.5f, s);
        q.y = __fmul_rn(__fadd_rn(yx, xy), s);
        q.z = __fmul_rn(__fadd_rn(xz, zx), s);
        q.w = __fmul_rn(__fsub_rn(zy, yz), s);
    } else if (yy > zz) {
        float s = (float)__dsqrt_rn(__dsub_rn(__dsub_rn(__dadd_rn(1.0, (double)yy), (double)xx), (double)zz));
        q.y = __fmul_rn(s, 0.5f);
        s = jdiv(0.5f, s);
        q.x = __fmul_rn(__fadd_rn(yx, xy), s);
        q.z = __fmul_rn(__fadd_rn(zy, yz), s);
        q.w = __fmul_rn(__fsub_rn(xz, zx), s);
    } else {
        float s = (float)__dsqrt_rn(__dsub_rn(__dsub_rn(__dadd_rn(1.0, (double)zz), (double)xx), (double)yy));
        q.z = __fmul_rn(s, 0.5f);
        s = jdiv(0.5f, s);
        q.x = __fmul_rn(__fadd_rn(xz, zx), s);
        q.y = __fmul_rn(__fadd_rn(zy, yz), s);
        q.w = __fmul_rn(__fsub_rn(yx, xy), s);
    }
    return q;
}
JBD M m_from_quat(Q q) {                // MatrixUtil.setRotation
    float d = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(q.x, q.x), __fmul_rn(q.y, q.y)), __fmul_rn(q.z, q.z)), __fmul_rn(q.w, q.w));
    float s = jdiv(2.0f, d);
    float xs = __fmul_rn(q.x, s), ys = __fmul_rn(q.y, s), zs = __fmul_rn(q.z, s);
    float wx = __fmul_rn(q.w, xs), wy = __fmul_rn(q.w, ys), wz = __fmul_rn(q.w, zs);
    float xx = __fmul_rn(q.x, xs), xy = __fmul_rn(q.x, ys), xz = __fmul_rn(q.x, zs);
    float yy = __fmul_rn(q.y, ys), yz = __fmul_rn(q.y, zs), zz = __fmul_rn(q.z, zs);
    M r;
    r.r[0] = mk(__fsub_rn(1.0f, __fadd_rn(yy, zz)), __fsub_rn(xy, wz), __fadd_rn(xz, wy));
    r.r[1] = mk(__fadd_rn(xy, wz), __fsub_rn(1.0f, __fadd_rn(xx, zz)), __fsub_rn(yz, wx));
    r.r[2] = mk(__fsub_rn(xz, wy), __fadd_rn(yz, wx), __fsub_rn(1.0f, __fadd_rn(xx, yy)));
    return r;
}
JBD Q q_axis_angle(V axis, float angle) {   // QuaternionUtil.setRotation
    float d = len(axis);
    float s = jdiv(jsin(__fmul_rn(angle, 0.5f)), d);
    Q q;
    q.x = __fmul_rn(axis.x, s); q.y = __fmul_rn(axis.y, s); q.z = __fmul_rn(axis.z, s);
    q.w = jcos(__fmul_rn(angle, 0.5f));
    return q;
}

constexpr float SIMDSQRT12 = 0.7071067811865475244008443621048490f;
JBD void plane_space1(V n, V& p, V& q) {    // TransformUtil.planeSpace1
    if (fabsf(n.z) > SIMDSQRT12) {
        float a = __fadd_rn(__fmul_rn(n.y, n.y), __fmul_rn(n.z, n.z));
        float k = jdiv(1.0f, jsqrt(a));
        p = mk(0.0f, __fmul_rn(-n.z, k), __fmul_rn(n.y, k));
        q = mk(__fmul_rn(a, k), __fmul_rn(-n.x, p.z), __fmul_rn(n.x, p.y));
    } else {
        float a = __fadd_rn(__fmul_rn(n.x, n.x), __fmul_rn(n.y, n.y));
        float k = jdiv(1.0f, jsqrt(a));
        p = mk(__fmul_rn(-n.y, k), __fmul_rn(n.x, k), 0.0f);
        q = mk(__fmul_rn(-n.z, p.y), __fmul_rn(n.z, p.x), __fmul_rn(a, k));
    }
}

// TransformUtil.integrateTransform
JBD Xf integrate_transform(const Xf& cur, V lin, V ang, float dt) {
    const float HALF_PI = __fmul_rn(SIMD_2_PI, 0.25f);
    const float THRESH = __fmul_rn(0.5f, HALF_PI);
    Xf p;
    p.o = mk(__fadd_rn(cur.o.x, __fmul_rn(dt, lin.x)), __fadd_rn(cur.o.y, __fmul_rn(dt, lin.y)),
             __fadd_rn(cur.o.z, __fmul_rn(dt, lin.z)));
    float fAngle = len(ang);
    if (__fmul_rn(fAngle, dt) > THRESH) fAngle = jdiv(THRESH, dt);
    V axis;
    if (fAngle < 0.001f) {
        float c = __fsub_rn(__fmul_rn(0.5f, dt),
                            __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(dt, dt), dt), 0.020833333333f), fAngle), fAngle));
        axis = scl(ang, c);
    } else {
        axis = scl(ang, jdiv(jsin(__fmul_rn(__fmul_rn(0.5f, fAngle), dt)), fAngle));
    }
    Q dorn;
    dorn.x = axis.x; dorn.y = axis.y; dorn.z = axis.z;
    dorn.w = jcos(__fmul_rn(__fmul_rn(fAngle, dt), 0.5f));
    Q orn0 = q_from_matrix(cur.b);
    Q pred = qnor(qmul(dorn, orn0));
    p.b = m_from_quat(pred);
    return p;
}

// TransformUtil.calculateVelocity / calculateDiffAxisAngle (linearmath/TransformUtil.java:105-153):
// the velocities that carry t0 to t1 in timeStep (QuaternionUtil.getAngle: 2 Math.acos(w)).
JBD void calc_velocity(const Xf& t0, const Xf& t1, float timeStep, V& lin, V& ang) {
    lin = scl(sub(t1.o, t0.o), jdiv(1.0f, timeStep));
    const Q dorn = qnor(q_from_matrix(mulMM(t1.b, m3_invert(t0.b))));
    const float angle = __fmul_rn(2.0f, (float)acos((double)dorn.w));
    V axis = mk(dorn.x, dorn.y, dorn.z);
    const float l2 = len2(axis);
    axis = l2 < __fmul_rn(FLT_EPS, FLT_EPS) ? mk(1.0f, 0.0f, 0.0f) : scl(axis, jdiv(1.0f, jsqrt(l2)));
    ang = scl(axis, jdiv(angle, timeStep));
}

}  // namespace jbd
