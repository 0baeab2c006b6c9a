// Which collision algorithm a pair runs, and on which two objects
// (collision/dispatch/CollisionDispatcher.findAlgorithm with DefaultCollisionConfiguration.
// getCollisionAlgorithmCreateFunc, java:160-215).  A pair with a compound body is stored once per
// child combination (key_sub): CompoundCollisionAlgorithm keeps one child algorithm per child
// and runs it with the child's shape at the body's transform times the child's
// (CompoundCollisionAlgorithm.java:49-67,83-127).  The compound's child comes first; with two
// compounds the child of the higher body does (the swapped algorithm the lower body's child
// finds against the higher compound puts its own child first).
#pragma once
#include "shapes.cuh"

namespace jbg {
using namespace jbd;

enum {
    ALG_EMPTY = 0,          // EmptyAlgorithm: two concave shapes (planes, meshes), no manifold
    ALG_SPHERE_SPHERE,      // SphereSphereCollisionAlgorithm
    ALG_CONVEX_PLANE,       // ConvexPlaneCollisionAlgorithm, convex first
    ALG_PLANE_CONVEX,       // the same, swapped
    ALG_CONVEX_CONVEX,      // ConvexConvexAlgorithm (GJK, EPA when penetrating)
    ALG_CONVEX_CONCAVE,     // ConvexConcaveCollisionAlgorithm, convex first
    ALG_CONCAVE_CONVEX      // the same, swapped
};

// An object as the algorithm sees it: shape index, world transform, body.
struct Leaf {
    int shape;
    Xf x;
    int body;
};

JBD int algorithm_kind(int tf, int tg) {
    if (tf == SHAPE_SPHERE && tg == SHAPE_SPHERE) return ALG_SPHERE_SPHERE;
    const bool cf = shape_is_convex(tf), cg = shape_is_convex(tg);
    if (cf && tg == SHAPE_PLANE) return ALG_CONVEX_PLANE;
    if (cg && tf == SHAPE_PLANE) return ALG_PLANE_CONVEX;
    if (cf && cg) return ALG_CONVEX_CONVEX;
    if (cf && shape_is_concave(tg)) return ALG_CONVEX_CONCAVE;
    if (cg && shape_is_concave(tf)) return ALG_CONCAVE_CONVEX;
    return ALG_EMPTY;
}

// CompoundShapeChild c's transform (basis rows, origin in .w).
JBD Xf child_xf(const DevShapes& sh, int c) {
    const float4 a = sh.child_xf[3 * c], b = sh.child_xf[3 * c + 1], d = sh.child_xf[3 * c + 2];
    Xf t;
    t.b.r[0] = mk(a.x, a.y, a.z);
    t.b.r[1] = mk(b.x, b.y, b.z);
    t.b.r[2] = mk(d.x, d.y, d.z);
    t.o = mk(a.w, b.w, d.w);
    return t;
}

// Child i of the compound shape s of a body at x: newChildWorldTrans.mul(orgTrans, childTrans).
JBD Leaf compound_child(const DevShapes& sh, int s, int i, const Xf& x, int body) {
    const int c = sh.child_off[s] + i;
    Leaf l;
    l.shape = sh.child_shape[c];
    l.x = xf_mul(x, child_xf(sh, c));
    l.body = body;
    return l;
}

// Child combinations of a pair of bodies (1 without compounds).
JBD int pair_subs(const DevShapes& sh, int s0, int s1) {
    return max(1, sh.child_cnt[s0]) * max(1, sh.child_cnt[s1]);
}

// The two objects of pair `key` between bodies col0 < col1 (root transforms x0, x1), in the
// algorithm's order, and the algorithm.
JBD int pair_leaves(const DevWorld& w, uint64_t key, int col0, int col1, const Xf& x0, const Xf& x1, Leaf& f, Leaf& g) {
    const int s0 = w.shape[col0], s1 = w.shape[col1];
    int tf = w.sh.type[s0], tg = w.sh.type[s1];
    f.shape = s0; f.x = x0; f.body = col0;
    g.shape = s1; g.x = x1; g.body = col1;
    if (tf == SHAPE_COMPOUND || tg == SHAPE_COMPOUND) {
        const int sub = key_sub(key);
        const int n1 = tg == SHAPE_COMPOUND ? w.sh.child_cnt[s1] : 1;
        const Leaf l0 = tf == SHAPE_COMPOUND ? compound_child(w.sh, s0, sub / n1, x0, col0) : f;
        const Leaf l1 = tg == SHAPE_COMPOUND ? compound_child(w.sh, s1, sub % n1, x1, col1) : g;
        if (tg == SHAPE_COMPOUND) { f = l1; g = l0; }
        else { f = l0; g = l1; }
        tf = w.sh.type[f.shape];
        tg = w.sh.type[g.shape];
    }
    return algorithm_kind(tf, tg);
}

// The leaf shape types only (no transforms): for grouping pairs by algorithm.
JBD int pair_leaf_types(const DevWorld& w, uint64_t key, int col0, int col1, int& tf, int& tg) {
    const int s0 = w.shape[col0], s1 = w.shape[col1];
    tf = w.sh.type[s0];
    tg = w.sh.type[s1];
    if (tf == SHAPE_COMPOUND || tg == SHAPE_COMPOUND) {
        const int sub = key_sub(key);
        const int n1 = tg == SHAPE_COMPOUND ? w.sh.child_cnt[s1] : 1;
        const int l0 = tf == SHAPE_COMPOUND ? w.sh.type[w.sh.child_shape[w.sh.child_off[s0] + sub / n1]] : tf;
        const int l1 = tg == SHAPE_COMPOUND ? w.sh.type[w.sh.child_shape[w.sh.child_off[s1] + sub % n1]] : tg;
        if (tg == SHAPE_COMPOUND) { tf = l1; tg = l0; }
        else { tf = l0; tg = l1; }
    }
    return algorithm_kind(tf, tg);
}

// OptimizedBvh.quantizeWithClamp (collision/shapes/OptimizedBvh.java:1038-1056) with a mesh's
// bvhAabbMin, bvhAabbMax and bvhQuantization.
JBD void mesh_quantize(V p, V bmin, V bmax, V q, int out[3]) {
    V c = mk(jmax(p.x, bmin.x), jmax(p.y, bmin.y), jmax(p.z, bmin.z));
    c = mk(jmin(c.x, bmax.x), jmin(c.y, bmax.y), jmin(c.z, bmax.z));
    V v = mulc(sub(c, bmin), q);
    out[0] = (int)__fadd_rn(v.x, 0.5f) & 0xFFFF;
    out[1] = (int)__fadd_rn(v.y, 0.5f) & 0xFFFF;
    out[2] = (int)__fadd_rn(v.z, 0.5f) & 0xFFFF;
}

// ConvexTriangleCallback's query of a convex leaf c against the mesh leaf t: c's box in the mesh's
// space widened by the mesh margin (setTimeStepAndCounters, ConvexTriangleCallback.java:82-104),
// quantized, and the mesh's tree walked as OptimizedBvh.walkStacklessQuantizedTree does
// (OptimizedBvh.java:940-997).  Returns the triangles found; the first `room` of them are written
// as (p, triangle) in walk order to out when out is given.
JBD int mesh_walk(const DevWorld& w, const Leaf& c, const Leaf& t, int p, int2* out, int room = 0) {
    const DevShapes& sh = w.sh;
    const Xf convexInTri = xf_mul(xf_inverse(t.x), c.x);
    V mn, mx;
    shape_aabb(sh, c.shape, convexInTri, mn, mx);
    const float mt = sh.margin[t.shape];
    mx = add(mx, mk(mt, mt, mt));
    mn = sub(mn, mk(mt, mt, mt));
    const float4* q = sh.mesh_q + 3 * t.shape;
    const V bmin = mk4(q[0]), bmax = mk4(q[1]), quant = mk4(q[2]);
    int qa[3], qb[3];
    mesh_quantize(mn, bmin, bmax, quant, qa);
    mesh_quantize(mx, bmin, bmax, quant, qb);
    const int4* nodes = sh.mesh_nodes + sh.mesh_node_off[t.shape];
    const int nn = sh.mesh_node_cnt[t.shape];
    int found = 0;
    for (int cur = 0; cur < nn;) {
        const int4 nd = nodes[cur];
        const int n0 = nd.x & 0xFFFF, n1 = (nd.x >> 16) & 0xFFFF, n2 = nd.y & 0xFFFF;
        const int m0 = (nd.y >> 16) & 0xFFFF, m1 = nd.z & 0xFFFF, m2 = (nd.z >> 16) & 0xFFFF;
        const bool ov = !(qa[0] > m0 || qb[0] < n0) && !(qa[2] > m2 || qb[2] < n2) && !(qa[1] > m1 || qb[1] < n1);
        const bool leaf = nd.w >= 0;
        if (leaf && ov) {
            if (out && found < room) out[found] = make_int2(p, nd.w & ((1 << 21) - 1));
            ++found;
        }
        cur += (ov || leaf) ? 1 : max(1, -nd.w);
    }
    return found;
}

// The triangle candidates the concave pass will list for body i against the listed mesh body m
// (every convex leaf of i: its compound children, or itself): the bound the pair count pass
// sums so that the candidate buffer is sized before the narrowphase.
JBD int mesh_candidates(const DevWorld& w, int i, int m) {
    const int si = w.shape[i], sm = w.shape[m];
    if (w.sh.type[sm] != SHAPE_MESH) return 0;
    Leaf t;
    t.shape = sm;
    t.x = load_xf(w, m);
    t.body = m;
    const Xf xi = load_xf(w, i);
    const int ti = w.sh.type[si];
    if (ti == SHAPE_COMPOUND) {
        int n = 0;
        for (int k = 0; k < w.sh.child_cnt[si]; k++) n += mesh_walk(w, compound_child(w.sh, si, k, xi, i), t, 0, nullptr);
        return n;
    }
    if (!shape_is_convex(ti)) return 0;
    Leaf c;
    c.shape = si;
    c.x = xi;
    c.body = i;
    return mesh_walk(w, c, t, 0, nullptr);
}

}  // namespace jbg
