// Persistent 4-point contact manifold on the device (collision/narrowphase/PersistentManifold.java,
// collision/dispatch/ManifoldResult.java of the reference).  A thread owns one pair's manifold,
// loads its points into registers/local memory, updates them and stores them back.
#pragma once
#include "jbgpu_internal.cuh"

namespace jbg {
using namespace jbd;

// A manifold point as the narrowphase sees it.  The fields it reads or recomputes every step are
// held here; the ones it only carries along (the lateral impulses, lateralFrictionInitialized and
// the two friction directions, which the solver writes) stay in memory: src is the slot the point
// came from in the stored manifold (-1 for a point added this step) and repl marks a point
// replaced in place (replaceContactPoint keeps its lateral impulses and directions and clears
// lateralFrictionInitialized), so that store_mf moves or resets them only when needed.
struct MP {
    V la, lb, wa, wb, n;
    float dist, fr, rest, ai;
    int life;
    int src;
    bool repl;
};
struct Mf {
    int n;
    MP p[4];
};

JBD void load_mf(const DevPairs& P, int pair, Mf& m) {
    m.n = P.n[pair];
    for (int j = 0; j < m.n; j++) {
        int k = pair * 4 + j;
        float4 a = P.pA[k], b = P.pB[k], c = P.wA[k], d = P.wB[k], e = P.nrm[k];
        MP& q = m.p[j];
        q.la = mk(a.x, a.y, a.z); q.dist = a.w;
        q.lb = mk(b.x, b.y, b.z); q.life = __float_as_int(b.w);
        q.wa = mk(c.x, c.y, c.z); q.fr = c.w;
        q.wb = mk(d.x, d.y, d.z); q.rest = d.w;
        q.n = mk(e.x, e.y, e.z); q.ai = e.w;
        q.src = j;
        q.repl = false;
    }
}
// Slots are written in increasing order; a moved point's source slot is never below its new slot
// (removeContactPoint moves the last point down), so a source is read before it is overwritten.
JBD void store_mf(const DevPairs& P, int pair, const Mf& m) {
    P.n[pair] = m.n;
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int j = 0; j < m.n; j++) {
        const int k = pair * 4 + j;
        const MP& q = m.p[j];
        const int s = pair * 4 + q.src;
        if (q.src < 0) {                           // added this step: no impulses, no directions
            P.imp[k] = zero;
            P.d1[k] = zero;
            P.d2[k] = zero;
        } else if (q.repl) {                       // replaced: impulses and directions kept, not initialised
            const float4 im = P.imp[s];
            if (q.src != j) { P.d1[k] = P.d1[s]; P.d2[k] = P.d2[s]; }
            P.imp[k] = make_float4(im.x, im.y, 0.0f, 0.0f);
        } else if (q.src != j) {                   // moved down by a removal
            P.imp[k] = P.imp[s];
            P.d1[k] = P.d1[s];
            P.d2[k] = P.d2[s];
        }
        P.pA[k] = f4(q.la, q.dist);
        P.pB[k] = f4(q.lb, __int_as_float(q.life));
        P.wA[k] = f4(q.wa, q.fr);
        P.wB[k] = f4(q.wb, q.rest);
        if (q.src != j || q.repl) P.nrm[k] = f4(q.n, q.ai);
    }
}

// PersistentManifold.sortCachedPoints (java:83-156) + VectorUtil.closestAxis4
JBD int sort_cached_points(const Mf& m, const MP& pt) {
    int maxPen = -1;
    float maxPenetration = pt.dist;
    for (int i = 0; i < 4; i++)
        if (m.p[i].dist < maxPenetration) { maxPen = i; maxPenetration = m.p[i].dist; }
    float r[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (maxPen != 0) r[0] = len2(crs(sub(pt.la, m.p[1].la), sub(m.p[3].la, m.p[2].la)));
    if (maxPen != 1) r[1] = len2(crs(sub(pt.la, m.p[0].la), sub(m.p[3].la, m.p[2].la)));
    if (maxPen != 2) r[2] = len2(crs(sub(pt.la, m.p[0].la), sub(m.p[3].la, m.p[1].la)));
    if (maxPen != 3) r[3] = len2(crs(sub(pt.la, m.p[0].la), sub(m.p[2].la, m.p[1].la)));
    int idx = -1;
    float best = -1e30f;
    for (int i = 0; i < 4; i++) {
        float v = fabsf(r[i]);
        if (v > best) { idx = i; best = v; }
    }
    return idx;
}

// PersistentManifold.removeContactPoint (java:259-278): the last point moves into the hole (the
// reference also clears the vacated slot's impulses and lifetime; the slot is past the count and
// is written in full before it is used again).
JBD void remove_point(Mf& m, int index) {
    int last = m.n - 1;
    if (index != last) m.p[index] = m.p[last];
    m.n--;
}

// PersistentManifold.refreshContactPoints (java:312-372) with the manifold bodies' transforms
JBD void refresh_points(Mf& m, const Xf& trA, const Xf& trB, float cbt) {
    for (int i = m.n - 1; i >= 0; i--) {
        MP& p = m.p[i];
        p.wa = xf_apply(trA, p.la);
        p.wb = xf_apply(trB, p.lb);
        p.dist = dot(sub(p.wa, p.wb), p.n);
        p.life++;
    }
    for (int i = m.n - 1; i >= 0; i--) {
        MP& p = m.p[i];
        if (!(p.dist <= cbt)) {
            remove_point(m, i);
        } else {
            V proj = sub(p.wa, scl(p.n, p.dist));
            V diff = sub(p.wb, proj);
            float d2 = dot(diff, diff);
            if (d2 > __fmul_rn(cbt, cbt)) remove_point(m, i);
        }
    }
}

// ManifoldResult.addContactPoint (java:92-157).  xf0/xf1 belong to col0/col1 (the pair's lower
// and higher uid); the manifold's body0 is mb0.
JBD void add_contact(Mf& m, int mb0, int col0, const Xf& xf0, const Xf& xf1, float fr0, float fr1, float re0, float re1,
                     V normalOnB, V pointInWorld, float depth, float cbt) {
    if (depth > cbt) return;
    bool swapped = mb0 != col0;
    V pointA = add(scl(normalOnB, depth), pointInWorld);
    V la, lb;
    if (swapped) { la = xf_invXform(xf1, pointA); lb = xf_invXform(xf0, pointInWorld); }
    else { la = xf_invXform(xf0, pointA); lb = xf_invXform(xf1, pointInWorld); }
    MP np;
    np.la = la; np.lb = lb; np.n = normalOnB; np.dist = depth;
    np.wa = pointA; np.wb = pointInWorld;
    np.ai = 0.0f; np.life = 0;
    np.src = -1;
    np.repl = false;
    float shortest = __fmul_rn(cbt, cbt);   // PersistentManifold.getCacheEntry (java:214-233)
    int nearest = -1;
    for (int i = 0; i < m.n; i++) {
        V d = sub(m.p[i].la, np.la);
        float dd = dot(d, d);
        if (dd < shortest) { shortest = dd; nearest = i; }
    }
    float fr = __fmul_rn(fr0, fr1);           // calculateCombinedFriction / Restitution (java:160-175)
    if (fr < -10.0f) fr = -10.0f;
    if (fr > 10.0f) fr = 10.0f;
    np.fr = fr;
    np.rest = __fmul_rn(re0, re1);
    if (nearest >= 0) {                       // replaceContactPoint keeps impulses and lifetime
        MP& o = m.p[nearest];
        const float ai = o.ai;
        const int life = o.life, src = o.src;
        o = np;
        o.ai = ai; o.life = life;
        o.src = src;                          // its lateral impulses and directions (store_mf)
        o.repl = true;
    } else {                                  // addManifoldPoint
        int ins = m.n;
        if (ins == 4) ins = sort_cached_points(m, np);
        else m.n++;
        m.p[ins] = np;
    }
}

}  // namespace jbg
