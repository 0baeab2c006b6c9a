// GJK closest points (collision/narrowphase/GjkPairDetector.java:73-316) with the Voronoi
// sub-simplex solver (collision/narrowphase/VoronoiSimplexSolver.java) on the device, one
// thread per convex pair.  The penetration fallback (GjkEpaSolver) lives in epa.cuh and
// runs in a second kernel over the pairs that need it.
#pragma once
#include "shapes.cuh"

namespace jbg {
using namespace jbd;

struct SubRes {
    V closest;
    bool uA, uB, uC, uD;
    float bc[4];
    bool degenerate;
};
JBD void sr_reset_used(SubRes& r) { r.uA = r.uB = r.uC = r.uD = false; }
JBD void sr_reset(SubRes& r) { r.degenerate = false; r.bc[0] = r.bc[1] = r.bc[2] = r.bc[3] = 0.0f; sr_reset_used(r); }
JBD bool sr_valid(const SubRes& r) { return r.bc[0] >= 0.0f && r.bc[1] >= 0.0f && r.bc[2] >= 0.0f && r.bc[3] >= 0.0f; }
JBD void sr_bc(SubRes& r, float a, float b, float c, float d) { r.bc[0] = a; r.bc[1] = b; r.bc[2] = c; r.bc[3] = d; }

// VoronoiSimplexSolver.closestPtPointTriangle (java:267-370), p = origin
JBD void closest_pt_triangle(V p, V a, V b, V c, SubRes& r) {
    sr_reset_used(r);
    V ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) { r.closest = a; r.uA = true; sr_bc(r, 1, 0, 0, 0); return; }
    V bp = sub(p, b);
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) { r.closest = b; r.uB = true; sr_bc(r, 0, 1, 0, 0); return; }
    float vc = __fsub_rn(__fmul_rn(d1, d4), __fmul_rn(d3, d2));
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = jdiv(d1, __fsub_rn(d1, d3));
        r.closest = mk(__fadd_rn(__fmul_rn(v, ab.x), a.x), __fadd_rn(__fmul_rn(v, ab.y), a.y), __fadd_rn(__fmul_rn(v, ab.z), a.z));
        r.uA = r.uB = true; sr_bc(r, __fsub_rn(1.0f, v), v, 0, 0); return;
    }
    V cp = sub(p, c);
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) { r.closest = c; r.uC = true; sr_bc(r, 0, 0, 1, 0); return; }
    float vb = __fsub_rn(__fmul_rn(d5, d2), __fmul_rn(d1, d6));
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float w = jdiv(d2, __fsub_rn(d2, d6));
        r.closest = mk(__fadd_rn(__fmul_rn(w, ac.x), a.x), __fadd_rn(__fmul_rn(w, ac.y), a.y), __fadd_rn(__fmul_rn(w, ac.z), a.z));
        r.uA = r.uC = true; sr_bc(r, __fsub_rn(1.0f, w), 0, w, 0); return;
    }
    float va = __fsub_rn(__fmul_rn(d3, d6), __fmul_rn(d5, d4));
    float d43 = __fsub_rn(d4, d3), d56 = __fsub_rn(d5, d6);
    if (va <= 0.0f && d43 >= 0.0f && d56 >= 0.0f) {
        float w = jdiv(d43, __fadd_rn(d43, d56));
        V t = sub(c, b);
        r.closest = mk(__fadd_rn(__fmul_rn(w, t.x), b.x), __fadd_rn(__fmul_rn(w, t.y), b.y), __fadd_rn(__fmul_rn(w, t.z), b.z));
        r.uB = r.uC = true; sr_bc(r, 0, __fsub_rn(1.0f, w), w, 0); return;
    }
    float denom = jdiv(1.0f, __fadd_rn(__fadd_rn(va, vb), vc));
    float v = __fmul_rn(vb, denom), w = __fmul_rn(vc, denom);
    V t1 = scl(ab, v), t2 = scl(ac, w);
    r.closest = mk(__fadd_rn(__fadd_rn(a.x, t1.x), t2.x), __fadd_rn(__fadd_rn(a.y, t1.y), t2.y), __fadd_rn(__fadd_rn(a.z, t1.z), t2.z));
    r.uA = r.uB = r.uC = true;
    sr_bc(r, __fsub_rn(__fsub_rn(1.0f, v), w), v, w, 0);
}

// VoronoiSimplexSolver.pointOutsideOfPlane (java:373-403)
JBD int point_outside_plane(V p, V a, V b, V c, V d) {
    V normal = crs(sub(b, a), sub(c, a));
    float signp = dot(sub(p, a), normal);
    float signd = dot(sub(d, a), normal);
    if (__fmul_rn(signd, signd) < __fmul_rn(1e-4f, 1e-4f)) return -1;
    return (__fmul_rn(signp, signd) < 0.0f) ? 1 : 0;
}

struct Simplex {
    int nv;
    V W[5], P[5], Q[5];
    V cP1, cP2, cV, lastW;
    bool valid, needsUpdate;
    SubRes bc;
};

JBD void sx_reset(Simplex& s) {
    s.valid = false;
    s.nv = 0;
    s.needsUpdate = true;
    s.lastW = mk(1e30f, 1e30f, 1e30f);
    sr_reset(s.bc);
    s.cP1 = s.cP2 = s.cV = mk(0.0f, 0.0f, 0.0f);
}
JBD void sx_remove(Simplex& s, int i) { s.nv--; s.W[i] = s.W[s.nv]; s.P[i] = s.P[s.nv]; s.Q[i] = s.Q[s.nv]; }
JBD void sx_reduce(Simplex& s, const SubRes& u) {
    if (s.nv >= 4 && !u.uD) sx_remove(s, 3);
    if (s.nv >= 3 && !u.uC) sx_remove(s, 2);
    if (s.nv >= 2 && !u.uB) sx_remove(s, 1);
    if (s.nv >= 1 && !u.uA) sx_remove(s, 0);
}
JBD bool sx_in(const Simplex& s, V w) {
    bool found = false;
    for (int i = 0; i < s.nv; i++) if (vequals(s.W[i], w)) found = true;
    if (vequals(w, s.lastW)) return true;
    return found;
}

// VoronoiSimplexSolver.closestPtPointTetrahedron (java:405-535), p = origin
JBD bool closest_pt_tetra(V a, V b, V c, V d, SubRes& fin) {
    V p = mk(0.0f, 0.0f, 0.0f);
    SubRes tmp;
    sr_reset(tmp);
    fin.closest = p;
    sr_reset_used(fin);
    fin.uA = fin.uB = fin.uC = fin.uD = true;
    int oABC = point_outside_plane(p, a, b, c, d);
    int oACD = point_outside_plane(p, a, c, d, b);
    int oADB = point_outside_plane(p, a, d, b, c);
    int oBDC = point_outside_plane(p, b, d, c, a);
    if (oABC < 0 || oACD < 0 || oADB < 0 || oBDC < 0) { fin.degenerate = true; return false; }
    if (oABC == 0 && oACD == 0 && oADB == 0 && oBDC == 0) return false;
    float best = 3.40282347e+38f;
    if (oABC != 0) {
        closest_pt_triangle(p, a, b, c, tmp);
        V t = sub(tmp.closest, p);
        float sq = dot(t, t);
        if (sq < best) {
            best = sq; fin.closest = tmp.closest; sr_reset_used(fin);
            fin.uA = tmp.uA; fin.uB = tmp.uB; fin.uC = tmp.uC;
            sr_bc(fin, tmp.bc[0], tmp.bc[1], tmp.bc[2], 0);
        }
    }
    if (oACD != 0) {
        closest_pt_triangle(p, a, c, d, tmp);
        V t = sub(tmp.closest, p);
        float sq = dot(t, t);
        if (sq < best) {
            best = sq; fin.closest = tmp.closest; sr_reset_used(fin);
            fin.uA = tmp.uA; fin.uC = tmp.uB; fin.uD = tmp.uC;
            sr_bc(fin, tmp.bc[0], 0, tmp.bc[1], tmp.bc[2]);
        }
    }
    if (oADB != 0) {
        closest_pt_triangle(p, a, d, b, tmp);
        V t = sub(tmp.closest, p);
        float sq = dot(t, t);
        if (sq < best) {
            best = sq; fin.closest = tmp.closest; sr_reset_used(fin);
            fin.uA = tmp.uA; fin.uB = tmp.uC; fin.uD = tmp.uB;
            sr_bc(fin, tmp.bc[0], tmp.bc[2], 0, tmp.bc[1]);
        }
    }
    if (oBDC != 0) {
        closest_pt_triangle(p, b, d, c, tmp);
        V t = sub(tmp.closest, p);
        float sq = dot(t, t);
        if (sq < best) {
            best = sq; fin.closest = tmp.closest; sr_reset_used(fin);
            fin.uB = tmp.uA; fin.uC = tmp.uC; fin.uD = tmp.uB;
            sr_bc(fin, 0, tmp.bc[0], tmp.bc[2], tmp.bc[1]);
        }
    }
    return true;
}

JBD V wsum3(V a, float x, V b, float y, V c, float z) {
    V t1 = scl(a, x), t2 = scl(b, y), t3 = scl(c, z);
    return mk(__fadd_rn(__fadd_rn(t1.x, t2.x), t3.x), __fadd_rn(__fadd_rn(t1.y, t2.y), t3.y), __fadd_rn(__fadd_rn(t1.z, t2.z), t3.z));
}

// VoronoiSimplexSolver.updateClosestVectorAndPoints (java:98-265)
JBD bool sx_update(Simplex& s) {
    if (s.needsUpdate) {
        sr_reset(s.bc);
        s.needsUpdate = false;
        switch (s.nv) {
        case 0:
            s.valid = false;
            break;
        case 1:
            s.cP1 = s.P[0];
            s.cP2 = s.Q[0];
            s.cV = sub(s.cP1, s.cP2);
            sr_reset(s.bc);
            sr_bc(s.bc, 1, 0, 0, 0);
            s.valid = sr_valid(s.bc);
            break;
        case 2: {
            V from = s.W[0], to = s.W[1];
            V diff = sub(mk(0.0f, 0.0f, 0.0f), from);
            V v = sub(to, from);
            float t = dot(v, diff);
            if (t > 0) {
                float dotVV = dot(v, v);
                if (t < dotVV) {
                    t = jdiv(t, dotVV);
                    diff = sub(diff, scl(v, t));
                    s.bc.uA = true; s.bc.uB = true;
                } else {
                    t = 1;
                    diff = sub(diff, v);
                    s.bc.uB = true;
                }
            } else {
                t = 0;
                s.bc.uA = true;
            }
            sr_bc(s.bc, __fsub_rn(1.0f, t), t, 0, 0);
            s.cP1 = add(s.P[0], scl(sub(s.P[1], s.P[0]), t));
            s.cP2 = add(s.Q[0], scl(sub(s.Q[1], s.Q[0]), t));
            s.cV = sub(s.cP1, s.cP2);
            sx_reduce(s, s.bc);
            s.valid = sr_valid(s.bc);
            break;
        }
        case 3: {
            closest_pt_triangle(mk(0.0f, 0.0f, 0.0f), s.W[0], s.W[1], s.W[2], s.bc);
            s.cP1 = wsum3(s.P[0], s.bc.bc[0], s.P[1], s.bc.bc[1], s.P[2], s.bc.bc[2]);
            s.cP2 = wsum3(s.Q[0], s.bc.bc[0], s.Q[1], s.bc.bc[1], s.Q[2], s.bc.bc[2]);
            s.cV = sub(s.cP1, s.cP2);
            sx_reduce(s, s.bc);
            s.valid = sr_valid(s.bc);
            break;
        }
        case 4: {
            bool sep = closest_pt_tetra(s.W[0], s.W[1], s.W[2], s.W[3], s.bc);
            if (sep) {
                V t1 = scl(s.P[0], s.bc.bc[0]), t2 = scl(s.P[1], s.bc.bc[1]), t3 = scl(s.P[2], s.bc.bc[2]), t4 = scl(s.P[3], s.bc.bc[3]);
                s.cP1 = mk(__fadd_rn(__fadd_rn(__fadd_rn(t1.x, t2.x), t3.x), t4.x), __fadd_rn(__fadd_rn(__fadd_rn(t1.y, t2.y), t3.y), t4.y),
                           __fadd_rn(__fadd_rn(__fadd_rn(t1.z, t2.z), t3.z), t4.z));
                t1 = scl(s.Q[0], s.bc.bc[0]); t2 = scl(s.Q[1], s.bc.bc[1]); t3 = scl(s.Q[2], s.bc.bc[2]); t4 = scl(s.Q[3], s.bc.bc[3]);
                s.cP2 = mk(__fadd_rn(__fadd_rn(__fadd_rn(t1.x, t2.x), t3.x), t4.x), __fadd_rn(__fadd_rn(__fadd_rn(t1.y, t2.y), t3.y), t4.y),
                           __fadd_rn(__fadd_rn(__fadd_rn(t1.z, t2.z), t3.z), t4.z));
                s.cV = sub(s.cP1, s.cP2);
                sx_reduce(s, s.bc);
            } else {
                if (s.bc.degenerate) s.valid = false;
                else { s.valid = true; s.cV = mk(0.0f, 0.0f, 0.0f); }
                break;
            }
            s.valid = sr_valid(s.bc);
            break;
        }
        default:
            s.valid = false;
        }
    }
    return s.valid;
}

// Result of the GJK part of GjkPairDetector.getClosestPoints, before the EPA fallback.
struct GjkPart {
    bool isValid;
    bool needEpa;    // checkPenetration && (!isValid || catchDegeneratePenetrationCase)
    float distance;
    V pointOnA, pointOnB, normalInB;
    V offset;        // positionOffset
};

// GjkPairDetector.getClosestPoints up to the penetration fallback (java:73-257)
JBD GjkPart gjk_part(const ShapeRef& sa, const Xf& tA, const ShapeRef& sb, const Xf& tB, float maxDist2) {
    const float REL_ERROR2 = 1.0e-6f;
    GjkPart r;
    r.distance = 0.0f;
    r.normalInB = mk(0.0f, 0.0f, 0.0f);
    r.pointOnA = r.pointOnB = mk(0.0f, 0.0f, 0.0f);
    r.offset = scl(add(tA.o, tB.o), 0.5f);
    Xf lA = tA, lB = tB;
    lA.o = sub(lA.o, r.offset);
    lB.o = sub(lB.o, r.offset);
    float marginA = sa.margin, marginB = sb.margin;
    int curIter = 0;
    V sep = mk(0.0f, 1.0f, 0.0f);
    bool isValid = false, checkSimplex = false, checkPenetration = true;
    int degenerate = 0;
    float sqd = SIMD_INFINITY;
    float margin = __fadd_rn(marginA, marginB);
    Simplex s;
    sx_reset(s);
    for (;;) {
        V sepA = mulMTv(scl(sep, -1.0f), tA.b);
        V sepB = mulMTv(sep, tB.b);
        V pInA = support_without_margin(sa, sepA);
        V qInB = support_without_margin(sb, sepB);
        V pW = xf_apply(lA, pInA);
        V qW = xf_apply(lB, qInB);
        V w = sub(pW, qW);
        float delta = dot(sep, w);
        if ((delta > 0.0f) && (__fmul_rn(delta, delta) > __fmul_rn(sqd, maxDist2))) { checkPenetration = false; break; }
        if (sx_in(s, w)) { degenerate = 1; checkSimplex = true; break; }
        float f0 = __fsub_rn(sqd, delta);
        float f1 = __fmul_rn(sqd, REL_ERROR2);
        if (f0 <= f1) { if (f0 <= 0.0f) degenerate = 2; checkSimplex = true; break; }
        s.lastW = w;                                 // addVertex
        s.needsUpdate = true;
        s.W[s.nv] = w; s.P[s.nv] = pW; s.Q[s.nv] = qW;
        s.nv++;
        bool ok = sx_update(s);                      // closest(v)
        sep = s.cV;
        if (!ok) { degenerate = 3; checkSimplex = true; break; }
        if (len2(sep) < REL_ERROR2) { degenerate = 6; checkSimplex = true; break; }
        float previous = sqd;
        sqd = len2(sep);
        if (__fsub_rn(previous, sqd) <= __fmul_rn(FLT_EPS, previous)) { sep = s.cV; checkSimplex = true; break; }
        if (curIter++ > 1000) break;
        if (s.nv == 4) { sep = s.cV; break; }
    }
    if (checkSimplex) {
        sx_update(s);                                // compute_points
        r.pointOnA = s.cP1;
        r.pointOnB = s.cP2;
        r.normalInB = sub(r.pointOnA, r.pointOnB);
        float lenSqr = len2(sep);
        if (lenSqr < 0.0001f) degenerate = 5;
        if (lenSqr > __fmul_rn(FLT_EPS, FLT_EPS)) {
            float rlen = jdiv(1.0f, jsqrt(lenSqr));
            r.normalInB = scl(r.normalInB, rlen);
            float sq = jsqrt(sqd);
            r.pointOnA = sub(r.pointOnA, scl(sep, jdiv(marginA, sq)));
            r.pointOnB = add(r.pointOnB, scl(sep, jdiv(marginB, sq)));
            r.distance = __fsub_rn(jdiv(1.0f, rlen), margin);
            isValid = true;
        }
    }
    bool catchDegen = (degenerate != 0 && (__fadd_rn(r.distance, margin) < 0.01f));
    r.isValid = isValid;
    r.needEpa = checkPenetration && (!isValid || catchDegen);
    return r;
}

}  // namespace jbg
