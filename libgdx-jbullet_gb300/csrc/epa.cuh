// Penetration depth by GJK + EPA (collision/narrowphase/GjkEpaSolver.java and
// GjkEpaPenetrationDepthSolver.java of the reference) on the device.  The polytope (faces,
// Minkowski vertices), the visited-ray set and the horizon stack live in a slot of a global
// scratch arena; the recursion of BuildHorizon runs on an explicit stack.
//
// One warp runs one query.  Every lane executes the whole (sequential) algorithm on identical
// values, so every lane reads back its own stores; the three scans — the best-face search, the
// visited-ray test and the hull support map — are split across the lanes and combined with warp
// shuffles under the reference's own selection rules, which gives the same result in every lane.
#pragma once
#include "gjk.cuh"

namespace jbg {
using namespace jbd;

constexpr int EPA_FACE_CAP = 1024;
constexpr int EPA_MKV_CAP = 288;
constexpr int EPA_SEEN_CAP = 136;
constexpr int EPA_STACK_CAP = 2 * EPA_FACE_CAP;

// The reference keeps the polytope's faces in a doubly linked list, newest first, and FindBest
// walks it for the first face of strictly smallest distance.  Faces enter the list only when
// created (prepended) and leave only through Detach, so the list is always the live faces in
// decreasing creation order: here a face is live when fE.w == 1, fD holds its distance (+inf
// once detached), and FindBest scans fD from the newest face down, which selects the same face.
struct EpaSlot {          // one query's polytope
    float4* fN;           // face normal xyz, distance w
    int4* fV;             // vertex ids, mark
    int4* fF;             // adjacent faces
    int4* fE;             // adjacent edges, live flag (w)
    float* fD;            // distance of live faces, +inf for faces outside the list
    float4* mW;           // Minkowski vertex w
    float4* mR;           // support direction r
    float4* seen;         // rays fetched by SearchOrigin (the reference's 64-bucket hash, as a set)
    int2* stack;          // BuildHorizon work list
    int faceCap, mkvCap, seenCap, stackCap;   // capacities (exceeding one sets the overflow flag)
};

struct EpaArena {
    float4 *fN, *mW, *mR, *seen;
    int4 *fV, *fF, *fE;
    float* fD;
    int2* stack;
    int slots;
};

JBD EpaSlot epa_slot(const EpaArena& a, int s) {
    EpaSlot e;
    e.fD = a.fD + (size_t)s * EPA_FACE_CAP;
    e.fN = a.fN + (size_t)s * EPA_FACE_CAP;
    e.fV = a.fV + (size_t)s * EPA_FACE_CAP;
    e.fF = a.fF + (size_t)s * EPA_FACE_CAP;
    e.fE = a.fE + (size_t)s * EPA_FACE_CAP;
    e.mW = a.mW + (size_t)s * EPA_MKV_CAP;
    e.mR = a.mR + (size_t)s * EPA_MKV_CAP;
    e.seen = a.seen + (size_t)s * EPA_SEEN_CAP;
    e.stack = a.stack + (size_t)s * EPA_STACK_CAP;
    e.faceCap = EPA_FACE_CAP;
    e.mkvCap = EPA_MKV_CAP;
    e.seenCap = EPA_SEEN_CAP;
    e.stackCap = EPA_STACK_CAP;
    return e;
}

struct EpaCtx {
    ShapeRef sh[2];
    M rot[2];
    V pos[2];
    float margin;
    V sw[5], sr[5];       // GJK simplex (Mkv w, r)
    V ray;
    int order, iterations, nseen;
    bool failed, overflow;
    EpaSlot sl;
    int nmkv, nface, root, nfaces;
    int lane, nl;         // lane in the warp and lanes sharing the query (1 or 32)
};

constexpr unsigned FULL_MASK = 0xffffffffu;

// support_with_margin with the hull's vertex scan split across nl lanes: each lane keeps the
// first strictly larger dot of its vertices, the warp then keeps the larger dot and, on equal
// dots, the lower vertex index — the vertex the sequential first-strict-maximum scan selects.
JBD V support_with_margin_lanes(const ShapeRef& s, V vec, int lane, int nl) {
    if (nl == 1 || s.type != SHAPE_HULL) return support_with_margin(s, vec);
    V v = normalize_dir(vec);
    float maxDot = -1e30f;
    int idx = 0x7fffffff;
    for (int i = lane; i < s.npts; i += 32) {
        float4 p = s.pts[i];
        float nd = dot(v, mk(p.x, p.y, p.z));
        if (nd > maxDot) { maxDot = nd; idx = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        float od = __shfl_xor_sync(FULL_MASK, maxDot, o);
        int oi = __shfl_xor_sync(FULL_MASK, idx, o);
        if (od > maxDot || (od == maxDot && oi < idx)) { maxDot = od; idx = oi; }
    }
    V sup = mk(0.0f, 0.0f, 0.0f);
    if (idx != 0x7fffffff) { float4 p = s.pts[idx]; sup = mk(p.x, p.y, p.z); }
    if (s.margin != 0.0f) {          // ConvexInternalShape.localGetSupportingVertex
        V vn = vec;
        if (len2(vn) < __fmul_rn(FLT_EPS, FLT_EPS)) vn = mk(-1.0f, -1.0f, -1.0f);
        vn = nor(vn);
        vn = scl(vn, s.margin);
        sup = add(sup, vn);
    }
    return sup;
}

JBD V epa_local_support(const EpaCtx& c, V d, int i) {     // GjkEpaSolver.GJK.LocalSupport
    V t = mulMTv(d, c.rot[i]);
    V o = support_with_margin_lanes(c.sh[i], t, c.lane, c.nl);
    o = mulMv(o, c.rot[i]);
    return add(o, c.pos[i]);
}
JBD void epa_support(const EpaCtx& c, V d, V& w, V& r) {    // GjkEpaSolver.GJK.Support
    r = d;
    V t1 = epa_local_support(c, d, 0);
    V t2 = epa_local_support(c, scl(d, -1.0f), 1);
    w = sub(t1, t2);
    w.x = __fadd_rn(w.x, __fmul_rn(c.margin, d.x));
    w.y = __fadd_rn(w.y, __fmul_rn(c.margin, d.y));
    w.z = __fadd_rn(w.z, __fmul_rn(c.margin, d.z));
}
JBD bool epa_fetch(EpaCtx& c) {                             // FetchSupport
    bool hit = false;
    for (int k = c.lane; k < c.nseen; k += c.nl) {
        float4 s = c.sl.seen[k];
        if (vequals(mk(s.x, s.y, s.z), c.ray)) hit = true;
    }
    if (c.nl > 1) hit = __any_sync(FULL_MASK, hit);
    if (hit) { --c.order; return false; }
    if (c.nseen < c.sl.seenCap) c.sl.seen[c.nseen++] = f4(c.ray, 0.0f);
    else c.overflow = true;
    ++c.order;
    epa_support(c, c.ray, c.sw[c.order], c.sr[c.order]);
    return dot(c.ray, c.sw[c.order]) > 0;
}
JBD void sx_copy(EpaCtx& c, int d, int s) { c.sw[d] = c.sw[s]; c.sr[d] = c.sr[s]; }

constexpr float GJK_INSIMPLEX_EPS = 0.0001f;

JBD bool epa_ss2(EpaCtx& c, V ao, V ab) {
    if (dot(ab, ao) >= 0) {
        V cabo = crs(ab, ao);
        if (len2(cabo) > __fmul_rn(GJK_INSIMPLEX_EPS, GJK_INSIMPLEX_EPS)) c.ray = crs(cabo, ab);
        else return true;
    } else {
        c.order = 0;
        sx_copy(c, 0, 1);
        c.ray = ao;
    }
    return false;
}
JBD bool epa_ss3a(EpaCtx& c, V ao, V ab, V ac, V cabc) {
    V t = crs(cabc, ab);
    V t2 = crs(cabc, ac);
    if (dot(t, ao) < -GJK_INSIMPLEX_EPS) {
        c.order = 1;
        sx_copy(c, 0, 1);
        sx_copy(c, 1, 2);
        return epa_ss2(c, ao, ab);
    } else if (dot(t2, ao) > +GJK_INSIMPLEX_EPS) {
        c.order = 1;
        sx_copy(c, 1, 2);
        return epa_ss2(c, ao, ac);
    } else {
        float d = dot(cabc, ao);
        if (fabsf(d) > GJK_INSIMPLEX_EPS) {
            if (d > 0) c.ray = cabc;
            else {
                c.ray = scl(cabc, -1.0f);
                V tw = c.sw[0], tr = c.sr[0];
                sx_copy(c, 0, 1);
                c.sw[1] = tw; c.sr[1] = tr;
            }
            return false;
        }
        return true;
    }
}
JBD bool epa_ss4(EpaCtx& c, V ao, V ab, V ac, V ad) {
    V t = crs(ab, ac), t2 = crs(ac, ad), t3 = crs(ad, ab);
    if (dot(t, ao) > GJK_INSIMPLEX_EPS) {
        c.order = 2;
        sx_copy(c, 0, 1); sx_copy(c, 1, 2); sx_copy(c, 2, 3);
        return epa_ss3a(c, ao, ab, ac, t);
    } else if (dot(t2, ao) > GJK_INSIMPLEX_EPS) {
        c.order = 2;
        sx_copy(c, 2, 3);
        return epa_ss3a(c, ao, ac, ad, t2);
    } else if (dot(t3, ao) > GJK_INSIMPLEX_EPS) {
        c.order = 2;
        sx_copy(c, 1, 0); sx_copy(c, 0, 2); sx_copy(c, 2, 3);
        return epa_ss3a(c, ao, ad, ab, t3);
    }
    return true;
}
JBD bool epa_search_origin(EpaCtx& c) {                     // GJK.SearchOrigin, initial ray (1,0,0)
    c.iterations = 0;
    c.order = -1;
    c.failed = false;
    c.ray = nor(mk(1.0f, 0.0f, 0.0f));
    c.nseen = 0;
    epa_fetch(c);
    c.ray = scl(c.sw[0], -1.0f);
    for (; c.iterations < 128; ++c.iterations) {
        float rl = len(c.ray);
        c.ray = scl(c.ray, jdiv(1.0f, rl > 0.0f ? rl : 1.0f));
        if (epa_fetch(c)) {
            bool found = false;
            if (c.order == 1) found = epa_ss2(c, scl(c.sw[1], -1.0f), sub(c.sw[0], c.sw[1]));
            else if (c.order == 2) found = epa_ss3a(c, scl(c.sw[2], -1.0f), sub(c.sw[1], c.sw[2]), sub(c.sw[0], c.sw[2]),
                                                   crs(sub(c.sw[1], c.sw[2]), sub(c.sw[0], c.sw[2])));
            else if (c.order == 3) found = epa_ss4(c, scl(c.sw[3], -1.0f), sub(c.sw[2], c.sw[3]), sub(c.sw[1], c.sw[3]),
                                                   sub(c.sw[0], c.sw[3]));
            if (found) return true;
        } else {
            return false;
        }
    }
    c.failed = true;
    return false;
}
JBD bool epa_enclose_origin(EpaCtx& c) {                    // GJK.EncloseOrigin
    if (c.order == 1) {
        V ab = sub(c.sw[1], c.sw[0]);
        // the reference evaluates b[i].set(ab).crs(b[i]) = ab x ab for all three axes
        V b = crs(ab, ab);
        Q q = q_axis_angle(nor(ab), jdiv(SIMD_2_PI, 3.0f));
        M r = m_from_quat(q);
        V w = b;
        epa_support(c, nor(w), c.sw[4], c.sr[4]);
        w = mulMv(w, r);
        epa_support(c, nor(w), c.sw[2], c.sr[2]);
        w = mulMv(w, r);
        epa_support(c, nor(w), c.sw[3], c.sr[3]);
        c.order = 4;
        return true;
    }
    if (c.order == 2) {
        V n = nor(crs(sub(c.sw[1], c.sw[0]), sub(c.sw[2], c.sw[0])));
        epa_support(c, n, c.sw[3], c.sr[3]);
        epa_support(c, scl(n, -1.0f), c.sw[4], c.sr[4]);
        c.order = 4;
        return true;
    }
    return c.order == 3 || c.order == 4;
}

// ---- EPA polytope ----------------------------------------------------------------------
__constant__ int c_mod3[5] = {0, 1, 2, 0, 1};
__constant__ int c_tet_f[4][3] = {{2, 1, 0}, {3, 0, 1}, {3, 1, 2}, {3, 2, 0}};
__constant__ int c_tet_e[6][4] = {{0, 0, 2, 1}, {0, 1, 1, 1}, {0, 2, 3, 1}, {1, 0, 3, 2}, {2, 0, 1, 2}, {3, 0, 2, 2}};
__constant__ int c_hex_f[6][3] = {{2, 0, 4}, {4, 1, 2}, {1, 4, 0}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
__constant__ int c_hex_e[9][4] = {{0, 0, 4, 0}, {0, 1, 2, 1}, {0, 2, 1, 2}, {1, 1, 5, 2}, {1, 0, 2, 0},
                                  {2, 2, 3, 2}, {3, 1, 5, 0}, {3, 0, 4, 2}, {5, 1, 4, 1}};

JBD int fget(int4 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
JBD void fset(int4& v, int i, int x) { if (i == 0) v.x = x; else if (i == 1) v.y = x; else v.z = x; }
JBD V mw(const EpaCtx& c, int i) { float4 a = c.sl.mW[i]; return mk(a.x, a.y, a.z); }

JBD int epa_new_mkv(EpaCtx& c, V w, V r) {
    if (c.nmkv >= c.sl.mkvCap) { c.overflow = true; return c.nmkv - 1; }
    c.sl.mW[c.nmkv] = f4(w, 0.0f);
    c.sl.mR[c.nmkv] = f4(r, 0.0f);
    return c.nmkv++;
}
JBD int epa_new_face(EpaCtx& c, int a, int b, int cc) {     // EPA.NewFace + EPA.Set
    if (c.nface >= c.sl.faceCap) { c.overflow = true; return c.nface - 1; }
    int id = c.nface++;
    V aw = mw(c, a), bw = mw(c, b), cw = mw(c, cc);
    V nrm = crs(sub(bw, aw), sub(cw, aw));
    float l = len(nrm);
    V t1 = crs(aw, bw), t2 = crs(bw, cw), t3 = crs(cw, aw);
    const float eps = 0.01f;
    bool valid = (dot(t1, nrm) >= -eps) && (dot(t2, nrm) >= -eps) && (dot(t3, nrm) >= -eps);
    V n = scl(nrm, jdiv(1.0f, l > 0.0f ? l : SIMD_INFINITY));
    float d = jmax(0.0f, -dot(n, aw));
    c.sl.fN[id] = f4(n, d);
    c.sl.fV[id] = make_int4(a, b, cc, 0);
    c.sl.fF[id] = make_int4(-1, -1, -1, 0);
    c.sl.fE[id] = make_int4(0, 0, 0, valid ? 1 : 0);   // prepended to the list when valid
    c.sl.fD[id] = valid ? d : __int_as_float(0x7f800000);
    if (valid) ++c.nfaces;
    return id;
}
// EPA.Detach: a listed face leaves the list unless it is the list's only face (then it has
// neither prev nor next and the reference's condition skips it).
JBD void epa_detach(EpaCtx& c, int f) {
    int4 E = c.sl.fE[f];
    if (E.w && c.nfaces > 1) {
        --c.nfaces;
        E.w = 0;
        c.sl.fE[f] = E;
        c.sl.fD[f] = __int_as_float(0x7f800000);
    }
}
JBD void epa_link(EpaCtx& c, int f0, int e0, int f1, int e1) {
    int4 F0 = c.sl.fF[f0], E0 = c.sl.fE[f0];
    fset(F0, e0, f1); fset(E0, e0, e1);
    c.sl.fF[f0] = F0; c.sl.fE[f0] = E0;
    int4 F1 = c.sl.fF[f1], E1 = c.sl.fE[f1];
    fset(F1, e1, f0); fset(E1, e1, e0);
    c.sl.fF[f1] = F1; c.sl.fE[f1] = E1;
}
JBD int epa_horizon(EpaCtx& c, int markid, int w, int f0, int e0, int& cf, int& ff) {   // EPA.BuildHorizon
    int ne = 0, sp = 0;
    c.sl.stack[sp++] = make_int2(f0, e0);
    V ww = mw(c, w);
    while (sp > 0) {
        int2 it = c.sl.stack[--sp];
        int f = it.x, e = it.y;
        int4 fv = c.sl.fV[f];
        if (fv.w == markid) continue;
        int e1 = c_mod3[e + 1];
        float4 fn = c.sl.fN[f];
        if (__fadd_rn(dot(mk(fn.x, fn.y, fn.z), ww), fn.w) > 0) {
            int nf = epa_new_face(c, fget(fv, e1), fget(fv, e), w);
            epa_link(c, nf, 0, f, e);
            if (cf >= 0) epa_link(c, cf, 1, nf, 2);
            else ff = nf;
            cf = nf;
            ne++;
        } else {
            int e2 = c_mod3[e + 2];
            epa_detach(c, f);
            fv.w = markid;
            c.sl.fV[f] = fv;
            int4 F = c.sl.fF[f], E = c.sl.fE[f];
            if (sp + 2 > c.sl.stackCap) { c.overflow = true; return ne; }
            c.sl.stack[sp++] = make_int2(fget(F, e2), fget(E, e2));
            c.sl.stack[sp++] = make_int2(fget(F, e1), fget(E, e1));
        }
    }
    return ne;
}

// GjkEpaSolver.collide -> EPA.EvaluatePD; returns true with witnesses on penetration.
JBD bool epa_pen_depth(const ShapeRef& s0, const Xf& t0, const ShapeRef& s1, const Xf& t1, EpaSlot slot, V& wA, V& wB,
                       bool& overflow, int lane, int nl) {
    EpaCtx c;
    c.lane = lane;
    c.nl = nl;
    c.sh[0] = s0; c.rot[0] = t0.b; c.pos[0] = t0.o;
    c.sh[1] = s1; c.rot[1] = t1.b; c.pos[1] = t1.o;
    c.margin = __fadd_rn(0.0f, 0.001f);
    c.sl = slot;
    c.overflow = false;
    c.nmkv = 0; c.nface = 0; c.root = -1; c.nfaces = 0;
    overflow = false;
    if (!epa_search_origin(c)) { overflow = c.overflow; return false; }
    // EvaluatePD(EPA_accuracy = 0.001)
    const float accuracy = 0.001f;
    int bestface = -1, markid = 1;
    float depth = -SIMD_INFINITY;
    if (epa_enclose_origin(c)) {
        int base = c.nmkv;
        for (int i = 0; i <= c.order; ++i) epa_new_mkv(c, c.sw[i], c.sr[i]);
        int bf[6];
        if (c.order == 3) {
            for (int i = 0; i < 4; i++) bf[i] = epa_new_face(c, base + c_tet_f[i][0], base + c_tet_f[i][1], base + c_tet_f[i][2]);
            for (int i = 0; i < 6; i++) epa_link(c, bf[c_tet_e[i][0]], c_tet_e[i][1], bf[c_tet_e[i][2]], c_tet_e[i][3]);
        } else if (c.order == 4) {
            for (int i = 0; i < 6; i++) bf[i] = epa_new_face(c, base + c_hex_f[i][0], base + c_hex_f[i][1], base + c_hex_f[i][2]);
            for (int i = 0; i < 9; i++) epa_link(c, bf[c_hex_e[i][0]], c_hex_e[i][1], bf[c_hex_e[i][2]], c_hex_e[i][3]);
        }
    }
    if (c.nfaces == 0) { overflow = c.overflow; return false; }   // depth = -inf, not > 0
    for (int it = 0; it < 256 && !c.overflow; ++it) {
        int best = -1;                                               // FindBest, newest face first
        {
            float bd = SIMD_INFINITY;
            for (int f = c.nface - 1 - c.lane; f >= 0; f -= c.nl) {
                float d = c.sl.fD[f];
                if (d < bd) { bd = d; best = f; }
            }
            if (c.nl > 1) {          // smallest distance; on equal distances the newer face
                for (int o = 16; o > 0; o >>= 1) {
                    float od = __shfl_xor_sync(FULL_MASK, bd, o);
                    int ob = __shfl_xor_sync(FULL_MASK, best, o);
                    if (od < bd || (od == bd && ob > best)) { bd = od; best = ob; }
                }
            }
        }
        if (best < 0) break;
        float4 bn = c.sl.fN[best];
        V n = mk(bn.x, bn.y, bn.z);
        V sw, sr;
        epa_support(c, scl(n, -1.0f), sw, sr);
        int w = epa_new_mkv(c, sw, sr);
        float d = __fadd_rn(dot(n, sw), bn.w);
        bestface = best;
        if (d < -accuracy) {
            int cf = -1, ff = -1, nf = 0;
            epa_detach(c, best);
            int4 fv = c.sl.fV[best];
            fv.w = ++markid;
            c.sl.fV[best] = fv;
            for (int i = 0; i < 3; ++i) {
                int4 F = c.sl.fF[best], E = c.sl.fE[best];
                nf += epa_horizon(c, markid, w, fget(F, i), fget(E, i), cf, ff);
            }
            if (nf <= 2) break;
            epa_link(c, cf, 1, ff, 2);
        } else {
            break;
        }
    }
    overflow = c.overflow;
    if (bestface < 0 || c.overflow) return false;
    float4 bn = c.sl.fN[bestface];
    int4 fv = c.sl.fV[bestface];
    int vi[3] = {fv.x, fv.y, fv.z};
    // GetCoordinates
    V o = scl(mk(bn.x, bn.y, bn.z), -bn.w);
    float a0 = len(crs(sub(mw(c, vi[0]), o), sub(mw(c, vi[1]), o)));
    float a1 = len(crs(sub(mw(c, vi[1]), o), sub(mw(c, vi[2]), o)));
    float a2 = len(crs(sub(mw(c, vi[2]), o), sub(mw(c, vi[0]), o)));
    float sm = __fadd_rn(__fadd_rn(a0, a1), a2);
    V b = scl(mk(a1, a2, a0), jdiv(1.0f, sm > 0.0f ? sm : 1.0f));
    depth = jmax(0.0f, bn.w);
    V nearest[2];
    for (int i = 0; i < 2; ++i) {
        float s = i != 0 ? -1.0f : 1.0f;
        V f[3];
        for (int j = 0; j < 3; ++j) {
            float4 r = c.sl.mR[vi[j]];
            f[j] = epa_local_support(c, scl(mk(r.x, r.y, r.z), s), i);
        }
        nearest[i] = wsum3(f[0], b.x, f[1], b.y, f[2], b.z);
    }
    if (depth > 0) {
        wA = nearest[0];
        wB = nearest[1];
        return true;
    }
    return false;
}

}  // namespace jbg
