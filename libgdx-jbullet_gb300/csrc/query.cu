// Scene queries: CollisionWorld.rayTest with a ClosestRayResultCallback for batches of rays
// (collision/dispatch/CollisionWorld.java:553-591, rayTestSingle 260-331,
// ClosestRayResultCallback 697-729).
//
// The reference walks every collision object in insertion order: the object's aabb against the
// ray (AabbUtil2.rayAabb, accepting entries up to the closest hit so far), then a
// SubsimplexConvexCast of a point along the ray (convex shapes) or the two triangles a
// StaticPlaneShape spans around the ray (TriangleRaycastCallback); a hit is taken when its
// fraction is below the closest so far.  Here one thread per ray walks the broadphase tree
// (refit over the shapes' current aabbs) twice - counting, then writing - to list every object
// whose aabb the ray enters before its end; then one thread per listed (ray, object) runs the
// object's cast, so that the warps run one code path (a thread per ray walking and casting by
// turns kept under two threads of a warp active).  An object's cast does not depend on the hits
// before it, so the ray's answer is its smallest hit by (fraction, body, triangle), j - found by
// a 64-bit atomicMin - unless an object before j in body order hit below j's aabb entry (then the
// order-dependent aabb test may have skipped j): such rays, rare, are replayed in body order by a
// block each.
#include "../../include/jbgpu.h"
#include "gjk.cuh"
#include "gridsync.cuh"
#include "prims.cuh"
#include "query.cuh"
#include "dispatch.cuh"
#include <climits>
#include "shapes.cuh"

namespace jbg {
using namespace jbd;

constexpr int RAY_STACK = 64;
constexpr int RAY_THREADS = 128;
constexpr int SLOW_THREADS = 256;

static inline int gridn(int n, int b) { return (n + b - 1) / b; }

__global__ void k_query_aabb(DevWorld w, float4* qmin, float4* qmax) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    V mn, mx;
    shape_aabb(w.sh, w.shape[i], load_xf(w, i), mn, mx);
    qmin[i] = f4(mn, 0.0f);
    qmax[i] = f4(mx, 0.0f);
}

// AabbUtil2.outcode (linearmath/AabbUtil2.java:40-43)
JBD int outcode(V p, V h) {
    return (p.x < -h.x ? 0x01 : 0x0) | (p.x > h.x ? 0x08 : 0x0) | (p.y < -h.y ? 0x02 : 0x0) | (p.y > h.y ? 0x10 : 0x0) |
           (p.z < -h.z ? 0x4 : 0x0) | (p.z > h.z ? 0x20 : 0x0);
}

// AabbUtil2.rayAabb (linearmath/AabbUtil2.java:45-104) split in two: the entry fraction and the
// exit bound of the box's planes (Math.min from +infinity).  The reference's test with param p
// passes iff the outcodes allow it and enter <= min(p, exit).
JBD bool ray_aabb_parts(V from, V to, V mn, V mx, float& enter, float& exit) {
    const V he = scl(sub(mx, mn), 0.5f);
    const V c = scl(add(mx, mn), 0.5f);
    const V source = sub(from, c), target = sub(to, c);
    const int so = outcode(source, he), tc = outcode(target, he);
    if ((so & tc) != 0) return false;
    enter = 0.0f;
    exit = __int_as_float(0x7f800000);
    const V r = sub(target, source);
    float normSign = 1.0f;
    int bit = 1;
    for (int j = 0; j < 2; j++) {
        for (int i = 0; i != 3; ++i) {
            if ((so & bit) != 0) {
                const float lambda = jdiv(__fsub_rn(-coord(source, i), __fmul_rn(coord(he, i), normSign)), coord(r, i));
                if (enter <= lambda) enter = lambda;
            } else if ((tc & bit) != 0) {
                const float lambda = jdiv(__fsub_rn(-coord(source, i), __fmul_rn(coord(he, i), normSign)), coord(r, i));
                exit = jmin(exit, lambda);
            }
            bit <<= 1;
        }
        normSign = -1.0f;
    }
    return true;
}

// VectorUtil.setInterpolate3 (linearmath/VectorUtil.java:137-144)
JBD V interp3(V a, V b, float rt) {
    const float s = __fsub_rn(1.0f, rt);
    return mk(__fadd_rn(__fmul_rn(s, a.x), __fmul_rn(rt, b.x)), __fadd_rn(__fmul_rn(s, a.y), __fmul_rn(rt, b.y)),
              __fadd_rn(__fmul_rn(s, a.z), __fmul_rn(rt, b.z)));
}

JBD M identity3() {
    M m;
    m.r[0] = mk(1.0f, 0.0f, 0.0f);
    m.r[1] = mk(0.0f, 1.0f, 0.0f);
    m.r[2] = mk(0.0f, 0.0f, 1.0f);
    return m;
}

// SubsimplexConvexCast.calcTimeOfImpact (collision/narrowphase/SubsimplexConvexCast.java:62-191)
// as rayTestSingle runs it: A is a sphere of radius 0 (its support is its centre) moving from the
// ray's start to its end with the identity basis, B the object's convex shape at rest.
JBD bool subsimplex_ray(const ShapeRef& sb, const Xf& tB, V from, V to, float& fraction, V& normal) {
    Simplex s;
    sx_reset(s);
    const V zero = mk(0.0f, 0.0f, 0.0f);
    Xf iA;
    iA.b = identity3();
    iA.o = from;
    const V linVelA = sub(to, from), linVelB = sub(tB.o, tB.o);
    float lambda = 0.0f;
    Xf iB = tB;
    const V r = sub(linVelA, linVelB);
    V supA = xf_apply(iA, zero);
    V supB = xf_apply(tB, support_with_margin(sb, mulMTv(r, tB.b)));
    V v = sub(supA, supB);
    int maxIter = 32;
    V n = zero;
    float dist2 = len2(v);
    while ((dist2 > 0.0001f) && (maxIter--) != 0) {
        supA = xf_apply(iA, zero);
        supB = xf_apply(iB, support_with_margin(sb, mulMTv(v, iB.b)));
        V w = sub(supA, supB);
        const float VdotW = dot(v, w);
        if (lambda > 1.0f) return false;
        if (VdotW > 0.0f) {
            const float VdotR = dot(v, r);
            if (VdotR >= -__fmul_rn(FLT_EPS, FLT_EPS)) return false;
            lambda = __fsub_rn(lambda, jdiv(VdotW, VdotR));
            iA.o = interp3(from, to, lambda);
            iB.o = interp3(tB.o, tB.o, lambda);
            w = sub(supA, supB);
            n = v;
        }
        s.lastW = w;                                 // addVertex
        s.needsUpdate = true;
        s.W[s.nv] = w; s.P[s.nv] = supA; s.Q[s.nv] = supB;
        s.nv++;
        const bool ok = sx_update(s);                // closest(v)
        v = s.cV;
        dist2 = ok ? len2(v) : 0.0f;
    }
    fraction = lambda;
    normal = len2(n) >= __fmul_rn(FLT_EPS, FLT_EPS) ? nor(n) : zero;
    return !(dot(normal, r) >= -0.0f);   // no time of impact when moving away (allowedPenetration 0)
}

// TriangleRaycastCallback.processTriangle (collision/narrowphase/TriangleRaycastCallback.java:
// 47-117) up to the report: the hit fraction and the local normal of a hit below `below`.
JBD bool ray_triangle(V t0, V t1, V t2, V from, V to, float below, float& distance, V& normal) {
    const V tn = crs(sub(t1, t0), sub(t2, t0));
    const float dist = dot(t0, tn);
    const float da = __fsub_rn(dot(tn, from), dist), db = __fsub_rn(dot(tn, to), dist);
    if (__fmul_rn(da, db) >= 0.0f) return false;
    distance = jdiv(da, __fsub_rn(da, db));
    if (!(distance < below)) return false;
    const float tol = __fmul_rn(len2(tn), -0.0001f);
    const V p = interp3(from, to, distance);
    const V v0p = sub(t0, p), v1p = sub(t1, p);
    if (!(dot(crs(v0p, v1p), tn) >= tol)) return false;
    const V v2p = sub(t2, p);
    if (!(dot(crs(v1p, v2p), tn) >= tol)) return false;
    if (!(dot(crs(v2p, v0p), tn) >= tol)) return false;
    normal = da > 0.0f ? tn : scl(tn, -1.0f);
    return true;
}

// rayTestSingle's compound branch (CollisionWorld.java:340-355): the convex branch on every child
// at the body's transform times the child's, in child order; the first smallest hit below 1 (the
// one the reference keeps, whatever closest fraction it enters with, whenever that hit wins).
JBD bool ray_compound(const DevShapes& sh, int s, const Xf& t, V from, V to, float& best, V& nrm) {
    best = 1.0f;
    bool hit = false;
    for (int i = 0, n = sh.child_cnt[s]; i < n; i++) {
        const int c = sh.child_off[s] + i;
        float f;
        V nl;
        if (subsimplex_ray(shape_ref(sh, sh.child_shape[c]), xf_mul(t, child_xf(sh, c)), from, to, f, nl) &&
            len2(nl) > 0.0001f && f < best) {
            best = f;
            nrm = nor(mulMv(nl, identity3()));
            hit = true;
        }
    }
    return hit;
}

// OptimizedBvh.walkStacklessQuantizedTreeAgainstRay (OptimizedBvh.java:817-938) in mesh shape s:
// the ray lf -> lt in the mesh's space, widened by a box cast's extents bmin / bmax (zero for a
// ray); a node is entered when its quantized box overlaps the query's quantized box and
// AabbUtil2.rayAabb with the bound 1 accepts its unquantized, widened box.  visit(tri) is called
// for every leaf entered, in walk order.
template <class Visit>
JBD void mesh_cast_walk(const DevShapes& sh, int s, V lf, V lt, V bmin, V bmax, Visit visit) {
    const float4* q = sh.mesh_q + 3 * s;
    const V qmin = mk4(q[0]), qmax = mk4(q[1]), quant = mk4(q[2]);
    int qa[3], qb[3];
    mesh_quantize(add(mk(jmin(lf.x, lt.x), jmin(lf.y, lt.y), jmin(lf.z, lt.z)), bmin), qmin, qmax, quant, qa);
    mesh_quantize(add(mk(jmax(lf.x, lt.x), jmax(lf.y, lt.y), jmax(lf.z, lt.z)), bmax), qmin, qmax, quant, qb);
    const int4* nodes = sh.mesh_nodes + sh.mesh_node_off[s];
    const int nn = sh.mesh_node_cnt[s];
    for (int cur = 0; cur < nn;) {
        const int4 nd = nodes[cur];
        const int n0 = nd.x & 0xFFFF, n1 = (nd.x >> 16) & 0xFFFF, n2 = nd.y & 0xFFFF;
        const int m0 = (nd.y >> 16) & 0xFFFF, m1 = nd.z & 0xFFFF, m2 = (nd.z >> 16) & 0xFFFF;
        const bool boxOv = !(qa[0] > m0 || qb[0] < n0) && !(qa[2] > m2 || qb[2] < n2) && !(qa[1] > m1 || qb[1] < n1);
        const bool leaf = nd.w >= 0;
        bool rayOv = false;
        if (boxOv) {
            const V b0 = add(add(mk(jdiv((float)n0, quant.x), jdiv((float)n1, quant.y), jdiv((float)n2, quant.z)), qmin), bmin);
            const V b1 = add(add(mk(jdiv((float)m0, quant.x), jdiv((float)m1, quant.y), jdiv((float)m2, quant.z)), qmin), bmax);
            float enter, exit;
            rayOv = ray_aabb_parts(lf, lt, b0, b1, enter, exit) && enter <= jmin(1.0f, exit);
        }
        if (leaf && rayOv) visit(nd.w & ((1 << 21) - 1));
        cur += (rayOv || leaf) ? 1 : max(1, -nd.w);
    }
}

// rayTestSingle's BvhTriangleMeshShape branch (CollisionWorld.java:297-311): the ray in the mesh's
// space through the walk without extents (reportRayOverlappingNodex), TriangleRaycastCallback on
// each leaf reached; the first smallest hit below 1, its normal times the mesh's basis.
JBD bool ray_mesh(const DevShapes& sh, int s, const Xf& t, V from, V to, float& best, V& nrm) {
    const Xf inv = xf_inverse(t);
    const V lf = xf_apply(inv, from), lt = xf_apply(inv, to);
    const V zero = mk(0.0f, 0.0f, 0.0f);
    const float4* tris = sh.mesh_tris + (size_t)3 * sh.mesh_tri_off[s];
    best = 1.0f;
    bool hit = false;
    mesh_cast_walk(sh, s, lf, lt, zero, zero, [&](int tri) {
        const float4* tv = tris + 3 * tri;
        float f;
        V nl;
        if (ray_triangle(mk4(tv[0]), mk4(tv[1]), mk4(tv[2]), lf, lt, best, f, nl)) {
            best = f;
            nrm = mulMv(nl, t.b);
            hit = true;
        }
    });
    return hit;
}

// SubsimplexConvexCast.calcTimeOfImpact (collision/narrowphase/SubsimplexConvexCast.java:62-191)
// for A moving from fromA to the origin toA (A's basis kept), B at rest at tB, allowedPenetration
// 0: the fraction, the unit normal and B's closest point (compute_points).
JBD bool subsimplex_cast(const ShapeRef& sa, const Xf& fromA, V toA, const ShapeRef& sb, const Xf& tB, float& fraction,
                         V& normal, V& hitPoint) {
    Simplex s;
    sx_reset(s);
    const V zero = mk(0.0f, 0.0f, 0.0f);
    Xf iA = fromA, iB = tB;
    const V r = sub(sub(toA, fromA.o), sub(tB.o, tB.o));
    V supA = xf_apply(fromA, support_with_margin(sa, mulMTv(scl(r, -1.0f), fromA.b)));
    V supB = xf_apply(tB, support_with_margin(sb, mulMTv(r, tB.b)));
    V v = sub(supA, supB);
    float lambda = 0.0f;
    int maxIter = 32;
    V n = zero;
    float dist2 = len2(v);
    while ((dist2 > 0.0001f) && (maxIter--) != 0) {
        supA = xf_apply(iA, support_with_margin(sa, mulMTv(scl(v, -1.0f), iA.b)));
        supB = xf_apply(iB, support_with_margin(sb, mulMTv(v, iB.b)));
        V w = sub(supA, supB);
        const float VdotW = dot(v, w);
        if (lambda > 1.0f) return false;
        if (VdotW > 0.0f) {
            const float VdotR = dot(v, r);
            if (VdotR >= -__fmul_rn(FLT_EPS, FLT_EPS)) return false;
            lambda = __fsub_rn(lambda, jdiv(VdotW, VdotR));
            iA.o = interp3(fromA.o, toA, lambda);
            iB.o = interp3(tB.o, tB.o, lambda);
            w = sub(supA, supB);
            n = v;
        }
        s.lastW = w;                                 // addVertex
        s.needsUpdate = true;
        s.W[s.nv] = w; s.P[s.nv] = supA; s.Q[s.nv] = supB;
        s.nv++;
        const bool ok = sx_update(s);                // closest(v)
        v = s.cV;
        dist2 = ok ? len2(v) : 0.0f;
    }
    fraction = lambda;
    normal = len2(n) >= __fmul_rn(FLT_EPS, FLT_EPS) ? nor(n) : zero;
    if (dot(normal, r) >= -0.0f) return false;
    sx_update(s);
    hitPoint = s.cP2;
    return true;
}

// objectQuerySingle's BvhTriangleMeshShape branch (CollisionWorld.java:425-455) for one mesh object
// at tM: the cast's origins in the mesh's space, widened by the cast shape's box (cbmin / cbmax: its
// aabb at the mesh-space rotation of its end transform), walked through the tree
// (reportBoxCastOverlappingNodex); each triangle reached is cast against by
// TriangleConvexcastCallback (SubsimplexConvexCast, |n|^2 > 1e-4) and accept(f, n, p) is offered
// every hit below 1 whose fraction is <= the last accepted one (BridgeTriangleConvexcastCallback.
// reportHit), in walk order; n is the cast's unit normal, which processTriangle normalises once
// more before reporting it (the caller does).
template <class Accept>
JBD void sweep_mesh(const DevShapes& sh, int s, const Xf& tM, const ShapeRef& cast, const Xf& from, V to, V cbmin,
                    V cbmax, Accept accept) {
    const Xf inv = xf_inverse(tM);
    const V lf = xf_apply(inv, from.o), lt = xf_apply(inv, to);
    float closest = 1.0f;
    mesh_cast_walk(sh, s, lf, lt, cbmin, cbmax, [&](int tri) {
        const ShapeRef tr = triangle_ref(sh, s, tri);
        float f;
        V n, p;
        if (!subsimplex_cast(cast, from, to, tr, tM, f, n, p)) return;
        if (!(len2(n) > 0.0001f) || !(f < 1.0f)) return;
        if (f <= closest && accept(f, n, p)) closest = f;
    });
}

// One object's part of rayTest with every hit below 1 (the bound of any closest fraction):
// rayTestSingle's convex branch (the normal rotated by the ray's identity basis and
// normalised) or its concave branch for a StaticPlaneShape, whose processAllTriangles
// (collision/shapes/StaticPlaneShape.java:60-120) spans two triangles around the ray's local
// aabb, taking half of the aabb's minimum corner as the half extent as the port does
// (halfExtents.set(aabbMax).set(aabbMin)).  Plane normals are the triangle normal times the
// object's basis (ClosestRayResultCallback with normalInWorldSpace false), not unit length.
struct ObjHits {
    int n;
    float f[2];
    V nrm[2];
};
JBD void ray_object(const DevWorld& w, int b, V from, V to, ObjHits& h) {
    h.n = 0;
    const int shape = w.shape[b];
    const Xf t = load_xf(w, b);
    if (w.sh.type[shape] == SHAPE_COMPOUND || w.sh.type[shape] == SHAPE_MESH) {
        float f;
        V n;
        if (w.sh.type[shape] == SHAPE_COMPOUND ? ray_compound(w.sh, shape, t, from, to, f, n)
                                               : ray_mesh(w.sh, shape, t, from, to, f, n)) {
            h.f[0] = f;
            h.nrm[0] = n;
            h.n = 1;
        }
        return;
    }
    if (w.sh.type[shape] != SHAPE_PLANE) {
        float f;
        V n;
        if (subsimplex_ray(shape_ref(w.sh, shape), t, from, to, f, n) && len2(n) > 0.0001f && f < 1.0f) {
            h.f[0] = f;
            h.nrm[0] = nor(mulMv(n, identity3()));
            h.n = 1;
        }
        return;
    }
    const float4 pl = w.sh.plane[shape];
    const V pn = mk(pl.x, pl.y, pl.z);
    const Xf inv = xf_inverse(t);
    const V lf = xf_apply(inv, from), lt = xf_apply(inv, to);
    const V mn = mk(jmin(lf.x, lt.x), jmin(lf.y, lt.y), jmin(lf.z, lt.z));
    const V mx = mk(jmax(lf.x, lt.x), jmax(lf.y, lt.y), jmax(lf.z, lt.z));
    const float radius = len(scl(mn, 0.5f));
    const V center = scl(add(mx, mn), 0.5f);
    V d0, d1;
    plane_space1(pn, d0, d1);
    const V pc = sub(center, scl(pn, __fsub_rn(dot(pn, center), pl.w)));
    const V a = scl(d0, radius), c = scl(d1, radius);
    const V amc = sub(a, c);
    float below = 1.0f;
    float dist;
    V nl;
    if (ray_triangle(add(add(pc, a), c), add(pc, amc), sub(pc, amc), lf, lt, below, dist, nl)) {
        h.f[h.n] = dist;
        h.nrm[h.n] = mulMv(nl, t.b);
        h.n++;
        below = dist;
    }
    if (ray_triangle(sub(pc, amc), sub(pc, add(a, c)), add(add(pc, a), c), lf, lt, below, dist, nl)) {
        h.f[h.n] = dist;
        h.nrm[h.n] = mulMv(nl, t.b);
        h.n++;
    }
}

JBD bool passes_filter(const DevWorld& w, int b, int group, int mask) {   // RayResultCallback.needsCollision
    return ((w.group[b] & mask) & 0xFFFF) != 0 && ((group & w.mask[b]) & 0xFFFF) != 0;
}

// Conservative slab test for the tree's inner boxes (inflated, so that no box the exact test
// accepts is culled).
JBD bool slab(V o, V d, float4 mn, float4 mx) {
    float tn = -1e-3f, tf = 1.001f;
    const float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    for (int k = 0; k < 3; k++) {
        const float e = 1e-4f * (1.0f + fmaxf(fabsf(lo[k]), fabsf(hi[k])));
        const float a = lo[k] - e, b = hi[k] + e;
        if (dd[k] == 0.0f) {
            if (oo[k] < a || oo[k] > b) return false;
            continue;
        }
        const float inv = 1.0f / dd[k];
        float t0 = (a - oo[k]) * inv, t1 = (b - oo[k]) * inv;
        if (t0 > t1) { const float x = t0; t0 = t1; t1 = x; }
        tn = fmaxf(tn, t0);
        tf = fminf(tf, t1);
        if (tn > tf) return false;
    }
    return true;
}

// A ray's candidate: a body whose aabb the ray enters before its end (rayAabb with the bound 1,
// which every closest fraction respects) and which passes the callback's filter.
struct RayCand {
    int ray, body;
    float enter;
    int pad;
};

// Tree walk of one ray per thread: COUNT counts the candidates, else they are written at the
// ray's offset (the same walk, so the same candidates in the same order).  GROW: a convex sweep's
// path of origins, every box (node and body) grown by the sweep's cast-shape box gmin / gmax.
template <bool COUNT, bool GROW = false>
__global__ void __launch_bounds__(RAY_THREADS) k_ray_walk(DevWorld w, DevWorld wq, const int* sortedBody, Bvh tree,
                                                         const int* wroot, const int* planeList, const int* planeStart,
                                                         const float* from, const float* to, const int* rayWorld, int n,
                                                         int nWorlds, int group, int mask, int* cnt, const int* off,
                                                         RayCand* cand, const float4* gmin = nullptr,
                                                         const float4* gmax = nullptr) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const V f = mk(from[3 * r], from[3 * r + 1], from[3 * r + 2]);
    const V t = mk(to[3 * r], to[3 * r + 1], to[3 * r + 2]);
    const int wi = rayWorld ? rayWorld[r] : 0;
    if (wi < 0 || wi >= nWorlds) {   // a world the batch does not have: no candidate, flagged
        if (COUNT) {
            cnt[r] = 0;
            atomicOr(&w.ctr[C_STATUS], ST_BAD_WORLD);
        }
        return;
    }
    const int base = COUNT ? 0 : off[r];
    const float4 g0 = GROW ? gmin[r] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 g1 = GROW ? gmax[r] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    int c = 0;
    auto consider = [&](int b) {
        if (!passes_filter(w, b, group, mask)) return;
        float enter, exit;
        const V bmin = GROW ? add(mk4(wq.amin[b]), mk4(g0)) : mk4(wq.amin[b]);
        const V bmax = GROW ? add(mk4(wq.amax[b]), mk4(g1)) : mk4(wq.amax[b]);
        if (!ray_aabb_parts(f, t, bmin, bmax, enter, exit)) return;
        if (!(enter <= jmin(1.0f, exit))) return;
        if (!COUNT) {
            RayCand rc;
            rc.ray = r;
            rc.body = b;
            rc.enter = enter;
            rc.pad = 0;
            cand[base + c] = rc;
        }
        c++;
    };
    const int root = wroot[wi];
    if (root != -1) {
        if (root & LEAF_FLAG) {
            consider(sortedBody[root & ~LEAF_FLAG]);
        } else {
            const V d = sub(t, f);
            int stack[RAY_STACK];
            int sp = 0;
            stack[sp++] = root;
            while (sp > 0) {
                const float4* nd = tree.node + 4 * stack[--sp];
                const float4 rec[4] = {nd[0], nd[1], nd[2], nd[3]};
                for (int k = 0; k < 2; k++) {
                    if (GROW) {
                        const float4 lo = rec[2 * k], hi = rec[2 * k + 1];
                        if (!slab(f, d, make_float4(__fadd_rn(lo.x, g0.x), __fadd_rn(lo.y, g0.y), __fadd_rn(lo.z, g0.z), 0.0f),
                                  make_float4(__fadd_rn(hi.x, g1.x), __fadd_rn(hi.y, g1.y), __fadd_rn(hi.z, g1.z), 0.0f)))
                            continue;
                    } else if (!slab(f, d, rec[2 * k], rec[2 * k + 1])) {
                        continue;
                    }
                    const int x = __float_as_int(rec[2 * k].w);
                    if (x & LEAF_FLAG) consider(sortedBody[x & ~LEAF_FLAG]);
                    else if (sp < RAY_STACK) stack[sp++] = x;
                    else atomicOr(&w.ctr[C_STATUS], ST_CAPACITY);
                }
            }
        }
    }
    for (int q = planeStart[wi]; q < planeStart[wi + 1]; q++) consider(planeList[q]);
    if (COUNT) cnt[r] = c;
}

JBD unsigned long long hit_key(float f, int body, int sub) {    // (fraction, body, triangle) order
    return ((unsigned long long)__float_as_uint(f) << 32) | ((unsigned long long)body << 1) | (unsigned)sub;
}

// One candidate per thread: the object's hits (ray_object), kept per candidate (.w = fraction,
// -1 for none), and the ray's smallest hit key by a 64-bit atomicMin (fractions are >= 0, so
// their bits order as the values do).
__global__ void __launch_bounds__(RAY_THREADS) k_ray_cast(DevWorld w, const RayCand* cand, int total, const float* from,
                                                         const float* to, float4* hitA, float4* hitB,
                                                         unsigned long long* key) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const RayCand c = cand[i];
    const V f = mk(from[3 * c.ray], from[3 * c.ray + 1], from[3 * c.ray + 2]);
    const V t = mk(to[3 * c.ray], to[3 * c.ray + 1], to[3 * c.ray + 2]);
    ObjHits h;
    ray_object(w, c.body, f, t, h);
    hitA[i] = h.n > 0 ? f4(h.nrm[0], h.f[0]) : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    hitB[i] = h.n > 1 ? f4(h.nrm[1], h.f[1]) : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
    for (int k = 0; k < h.n; k++) atomicMin(key + c.ray, hit_key(h.f[k], c.body, k));
}

// The candidate holding a ray's smallest hit j writes the ray's record and j's aabb entry.
__global__ void k_ray_pick(const RayCand* cand, int total, const float4* hitA, const float4* hitB,
                           const unsigned long long* key, const float* from, const float* to, float* enterJ,
                           jbgpu_ray_hit* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const RayCand c = cand[i];
    const unsigned long long k = key[c.ray];
    if (k == ~0ull || (int)((k >> 1) & 0x7fffffffu) != c.body) return;
    const float4 h = (k & 1) ? hitB[i] : hitA[i];
    enterJ[c.ray] = c.enter;
    jbgpu_ray_hit o;
    o.body = c.body;
    o.fraction = h.w;
    o.normal[0] = h.x; o.normal[1] = h.y; o.normal[2] = h.z;
    const V p = interp3(mk(from[3 * c.ray], from[3 * c.ray + 1], from[3 * c.ray + 2]),
                        mk(to[3 * c.ray], to[3 * c.ray + 1], to[3 * c.ray + 2]), h.w);
    o.point[0] = p.x; o.point[1] = p.y; o.point[2] = p.z;
    out[c.ray] = o;
}

// j is the reference's answer unless an object before it in body order hit below j's aabb
// entry (the reference's aabb test, bounded by the closest hit so far, could then skip j).
__global__ void k_ray_check(const RayCand* cand, int total, const float4* hitA, const float4* hitB,
                            const unsigned long long* key, const float* enterJ, int* undecided) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const RayCand c = cand[i];
    const unsigned long long k = key[c.ray];
    if (k == ~0ull || c.body >= (int)((k >> 1) & 0x7fffffffu)) return;
    const float e = enterJ[c.ray];
    const float a = hitA[i].w, b = hitB[i].w;
    if ((a >= 0.0f && a < e) || (b >= 0.0f && b < e)) undecided[c.ray] = 1;
}

// Rays without a hit get the callback's untouched record; undecided rays (and every ray when
// the replay is forced) go to the in-order replay.
__global__ void k_ray_finish(int n, const unsigned long long* key, const int* undecided, int replayAll,
                             jbgpu_ray_hit* out, int* slow, int* slowCount) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    if (replayAll || undecided[r]) {
        slow[atomicAdd(slowCount, 1)] = r;
        return;
    }
    if (key[r] != ~0ull) return;
    jbgpu_ray_hit o;
    o.body = -1;
    o.fraction = 1.0f;
    o.normal[0] = o.normal[1] = o.normal[2] = 0.0f;
    o.point[0] = o.point[1] = o.point[2] = 0.0f;
    out[r] = o;
}

// The reference's loop for the undecided rays, a block per ray: every body of the ray's world in
// index order, a chunk of SLOW_THREADS at a time evaluated in parallel (the aabb parts and the
// object's hits do not depend on the closest fraction), then replayed by one thread with the
// closest fraction and the break at zero.
__global__ void __launch_bounds__(SLOW_THREADS) k_rays_slow(DevWorld w, DevWorld wq, const float* from, const float* to,
                                                          const int* rayWorld, int group, int mask, jbgpu_ray_hit* out,
                                                          const int* slow, const int* slowCount) {
    __shared__ int sOk[SLOW_THREADS];
    __shared__ float sEnter[SLOW_THREADS], sExit[SLOW_THREADS];
    __shared__ ObjHits sHits[SLOW_THREADS];
    __shared__ int sStop;
    const int count = *slowCount;
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const int r = slow[q];
        const V f = mk(from[3 * r], from[3 * r + 1], from[3 * r + 2]);
        const V t = mk(to[3 * r], to[3 * r + 1], to[3 * r + 2]);
        const int wi = rayWorld ? rayWorld[r] : 0;
        float closest = 1.0f;
        int body = -1;
        V normal = mk(0.0f, 0.0f, 0.0f);
        if (threadIdx.x == 0) sStop = 0;
        __syncthreads();
        for (int base = 0; base < w.nBodies; base += SLOW_THREADS) {
            const int b = base + threadIdx.x;
            int ok = 0;
            if (b < w.nBodies && w.world[b] == wi && passes_filter(w, b, group, mask)) {
                float enter, exit;
                if (ray_aabb_parts(f, t, mk4(wq.amin[b]), mk4(wq.amax[b]), enter, exit) && enter <= jmin(1.0f, exit)) {
                    ok = 1;
                    sEnter[threadIdx.x] = enter;
                    sExit[threadIdx.x] = exit;
                    ray_object(w, b, f, t, sHits[threadIdx.x]);
                }
            }
            sOk[threadIdx.x] = ok;
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int k = 0; k < SLOW_THREADS && base + k < w.nBodies; k++) {
                    if (closest == 0.0f) { sStop = 1; break; }
                    if (!sOk[k] || !(sEnter[k] <= jmin(closest, sExit[k]))) continue;
                    const ObjHits& h = sHits[k];
                    for (int m = 0; m < h.n; m++)
                        if (h.f[m] < closest) {
                            closest = h.f[m];
                            body = base + k;
                            normal = h.nrm[m];
                        }
                }
            }
            __syncthreads();
            if (sStop) break;
        }
        if (threadIdx.x == 0) {
            jbgpu_ray_hit o;
            o.body = body;
            o.fraction = closest;
            o.normal[0] = normal.x; o.normal[1] = normal.y; o.normal[2] = normal.z;
            const V p = body >= 0 ? interp3(f, t, closest) : mk(0.0f, 0.0f, 0.0f);
            o.point[0] = p.x; o.point[1] = p.y; o.point[2] = p.z;
            out[r] = o;
        }
        __syncthreads();
    }
}

// ---- convexSweepTest ------------------------------------------------------------------------
// CollisionWorld.convexSweepTest with a ClosestConvexResultCallback (collision/dispatch/
// CollisionWorld.java:596-645, objectQuerySingle 391-490).  The reference's object loop tests each
// object's aabb, grown by the cast shape's temporal aabb, against the path of the origins with
// the fixed bound 1 and keeps a GjkConvexCast hit when it is below the closest so far: the answer
// is the smallest hit by (fraction, body), whatever the order.  The rays' tree walk, with every
// box grown by the cast shape's box, lists the (sweep, body) candidates; a thread per candidate
// casts.

JBD Xf xf12(const float* f) {
    Xf t;
    t.b.r[0] = mk(f[0], f[1], f[2]);
    t.b.r[1] = mk(f[3], f[4], f[5]);
    t.b.r[2] = mk(f[6], f[7], f[8]);
    t.o = mk(f[9], f[10], f[11]);
    return t;
}

// The box a cast shape sweeps from transform f to t, as convexSweepTest forms it:
// TransformUtil.calculateVelocity / calculateDiffAxisAngle (linearmath/TransformUtil.java:105-153)
// and CollisionShape.calculateTemporalAabb with getAngularMotionDisc (CollisionShape.java:44-121),
// at the start rotation.  aabb(x, mn, mx) is the cast shape's getAabb.
template <class AabbFn>
JBD void cast_box(const Xf& f, const Xf& t, AabbFn aabb, V& cmin, V& cmax) {
    const V linVel = scl(sub(t.o, f.o), jdiv(1.0f, 1.0f));
    const Q dorn = qnor(q_from_matrix(mulMM(t.b, m3_invert(f.b))));
    const float angle = __fmul_rn(2.0f, (float)acos((double)dorn.w));
    V axis = mk(dorn.x, dorn.y, dorn.z);
    const float l2 = len2(axis);
    axis = l2 < __fmul_rn(FLT_EPS, FLT_EPS) ? mk(1.0f, 0.0f, 0.0f) : scl(axis, jdiv(1.0f, jsqrt(l2)));
    const V angVel = scl(axis, jdiv(angle, 1.0f));
    Xf R;
    R.b = m_from_quat(q_from_matrix(f.b));
    R.o = mk(0.0f, 0.0f, 0.0f);
    V mn, mx;
    aabb(R, mn, mx);
    const V lin = scl(linVel, 1.0f);
    if (lin.x > 0.0f) mx.x = __fadd_rn(mx.x, lin.x); else mn.x = __fadd_rn(mn.x, lin.x);
    if (lin.y > 0.0f) mx.y = __fadd_rn(mx.y, lin.y); else mn.y = __fadd_rn(mn.y, lin.y);
    if (lin.z > 0.0f) mx.z = __fadd_rn(mx.z, lin.z); else mn.z = __fadd_rn(mn.z, lin.z);
    Xf I;
    I.b.r[0] = mk(1.0f, 0.0f, 0.0f); I.b.r[1] = mk(0.0f, 1.0f, 0.0f); I.b.r[2] = mk(0.0f, 0.0f, 1.0f);
    I.o = mk(0.0f, 0.0f, 0.0f);
    V bmin, bmax;
    aabb(I, bmin, bmax);
    const float radius = __fmul_rn(len(sub(bmax, bmin)), 0.5f);
    const float disc = __fadd_rn(radius, len(scl(add(bmin, bmax), 0.5f)));
    const float am = __fmul_rn(__fmul_rn(len(angVel), disc), 1.0f);
    cmin = sub(mn, mk(am, am, am));
    cmax = add(mx, mk(am, am, am));
}

__global__ void k_sweep_prep(DevWorld w, int shape, const float* from, const float* to, int n, float4* cmin,
                             float4* cmax, float* ofrom, float* oto) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float* f = from + 12 * q;
    const float* t = to + 12 * q;
    for (int k = 0; k < 3; k++) {   // the path of the origins, walked like a ray
        ofrom[3 * q + k] = f[9 + k];
        oto[3 * q + k] = t[9 + k];
    }
    V mn, mx;
    cast_box(xf12(f), xf12(t), [&](const Xf& x, V& a, V& b) { shape_aabb(w.sh, shape, x, a, b); }, mn, mx);
    cmin[q] = f4(mn, 0.0f);
    cmax[q] = f4(mx, 0.0f);
}

// GjkConvexCast.calcTimeOfImpact (collision/narrowphase/GjkConvexCast.java:67-185): conservative
// advancement on GjkPairDetector distances without a penetration solver, through a PointCollector
// that keeps its closest result across the calls.
JBD bool gjk_convex_cast(const ShapeRef& sa, const Xf& fromA, V toA, const ShapeRef& sb, const Xf& tB, float& fraction,
                         V& normal, V& hitPoint) {
    const V r = sub(sub(toA, fromA.o), sub(tB.o, tB.o));
    float lambda = 0.0f, lastLambda = 0.0f;
    int numIter = 0;
    bool has = false;
    float cdist = 1e30f;
    V cn = mk(0.0f, 0.0f, 0.0f), cp = cn;
    Xf iA = fromA, iB = tB;
    auto collect = [&]() {
        const GjkPart g = gjk_part(sa, iA, sb, iB, SIMD_INFINITY);
        if (g.isValid && g.distance < cdist) {
            has = true;
            cn = g.normalInB;
            cp = add(g.pointOnB, g.offset);
            cdist = g.distance;
        }
    };
    collect();
    if (!has) return false;
    V c = cp, n = cn;
    float dist = cdist;
    while (dist > 0.001f) {
        if (++numIter > 32) return false;
        lambda = __fsub_rn(lambda, jdiv(dist, dot(r, n)));
        if (lambda > 1.0f || lambda < 0.0f || lambda <= lastLambda) return false;
        lastLambda = lambda;
        iA.o = interp3(fromA.o, toA, lambda);
        iB.o = interp3(tB.o, tB.o, lambda);
        collect();
        if (cdist < 0.0f) { fraction = lastLambda; normal = cn; hitPoint = cp; return true; }
        c = cp;
        n = cn;
        dist = cdist;
    }
    if (dot(n, r) >= -0.04f) return false;   // DispatcherInfo.allowedCcdPenetration
    fraction = lambda;
    normal = n;
    hitPoint = c;
    return true;
}

int query_prepare(const DevWorld& w, BroadphaseBuffers& bb, QueryBuffers& qb, cudaStream_t s) {
    if (w.nBodies > qb.capBodies) {
        if (qb.qmin) cudaFree(qb.qmin);
        if (qb.qmax) cudaFree(qb.qmax);
        qb.qmin = qb.qmax = nullptr;
        qb.capBodies = 0;
        const int c = w.nBodies > 2 * qb.capBodies ? w.nBodies : 2 * qb.capBodies;
        if (cudaMalloc((void**)&qb.qmin, sizeof(float4) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.qmax, sizeof(float4) * (size_t)c) != cudaSuccess)
            return JBGPU_ERR_CUDA;
        qb.capBodies = c;
    }
    if (w.nBodies == 0) return JBGPU_OK;
    k_query_aabb<<<gridn(w.nBodies, 256), 256, 0, s>>>(w, qb.qmin, qb.qmax); note_launch();
    DevWorld wq = w;
    wq.amin = qb.qmin;
    wq.amax = qb.qmax;
    if (!bb.built) broadphase_build_tree(wq, bb, s);
    const int nodes = bb.nFinite > 1 ? bb.nFinite - 1 : 1;
    if (nodes > qb.capNodes) {
        if (qb.node) cudaFree(qb.node);
        if (qb.visit) cudaFree(qb.visit);
        qb.node = nullptr;
        qb.visit = nullptr;
        const int c = nodes > 2 * qb.capNodes ? nodes : 2 * qb.capNodes;
        qb.capNodes = 0;
        if (cudaMalloc((void**)&qb.node, sizeof(float4) * 4 * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.visit, sizeof(int) * (size_t)c) != cudaSuccess)
            return JBGPU_ERR_CUDA;
        qb.capNodes = c;
    }
    broadphase_refit_into(wq, bb, qb.node, qb.visit, s);
    return cudaGetLastError() == cudaSuccess ? JBGPU_OK : JBGPU_ERR_CUDA;
}

static bool grow_ray_buffers(QueryBuffers& qb, int n) {
    if (n > qb.capRays) {   // per-ray (per-sweep) buffers
        void* old[] = {qb.slow, qb.rayCnt, qb.rayOff, qb.key, qb.enterJ, qb.undecided, qb.scanScratch};
        for (void* p : old)
            if (p) cudaFree(p);
        qb.slow = qb.rayCnt = qb.rayOff = qb.undecided = nullptr;
        qb.key = nullptr;
        qb.enterJ = nullptr;
        qb.scanScratch = nullptr;
        const int c = n > 2 * qb.capRays ? n : 2 * qb.capRays;
        qb.capRays = 0;
        if (cudaMalloc((void**)&qb.slow, sizeof(int) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.rayCnt, sizeof(int) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.rayOff, sizeof(int) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.key, sizeof(unsigned long long) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.enterJ, sizeof(float) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.undecided, sizeof(int) * (size_t)c) != cudaSuccess ||
            cudaMalloc(&qb.scanScratch, scan_scratch_bytes(c)) != cudaSuccess)
            return false;
        qb.capRays = c;
    }
    if (!qb.slowCount && (cudaMalloc((void**)&qb.slowCount, sizeof(int)) != cudaSuccess ||
                          cudaMalloc((void**)&qb.candTotal, sizeof(int)) != cudaSuccess ||
                          cudaMalloc((void**)&qb.candTotal64, sizeof(unsigned long long)) != cudaSuccess))
        return false;
    return true;
}

static bool grow_cand_buffers(QueryBuffers& qb, int total) {
    if (total > qb.capCand) {
        void* old[] = {qb.cand, qb.hitA, qb.hitB};
        for (void* p : old)
            if (p) cudaFree(p);
        qb.cand = nullptr;
        qb.hitA = qb.hitB = nullptr;
        const int c = total > 2 * qb.capCand ? total : 2 * qb.capCand;
        qb.capCand = 0;
        if (cudaMalloc((void**)&qb.cand, sizeof(RayCand) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.hitA, sizeof(float4) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.hitB, sizeof(float4) * (size_t)c) != cudaSuccess)
            return false;
        qb.capCand = c;
    }
    return true;
}

// 64-bit sum of the walk's per-ray candidate counts: the int scan that places the candidates is
// only used when this total fits in an int.
__global__ void k_total64(const int* cnt, int n, unsigned long long* total) {
    unsigned long long v = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v += (unsigned)cnt[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(total, v);
}

// The candidate total of a walk (per-ray counts already scanned into qb.candTotal): summed again
// in 64 bits, so that a batch whose (ray, body) candidates do not fit in an int is refused
// (JBGPU_ERR_CAPACITY: split the batch) instead of wrapping.
static int candidate_total(QueryBuffers& qb, int n, cudaStream_t s, int& total) {
    cudaMemsetAsync(qb.candTotal64, 0, sizeof(unsigned long long), s);
    const int blocks = gridn(n, 256) < 1024 ? gridn(n, 256) : 1024;
    k_total64<<<blocks, 256, 0, s>>>(qb.rayCnt, n, qb.candTotal64);
    note_launch();
    unsigned long long t64 = 0;
    if (cudaMemcpyAsync(&total, qb.candTotal, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&t64, qb.candTotal64, sizeof(t64), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return JBGPU_ERR_CUDA;
    if (t64 > (unsigned long long)INT_MAX) return JBGPU_ERR_CAPACITY;
    return JBGPU_OK;
}

int query_rays(const DevWorld& w, const BroadphaseBuffers& bb, QueryBuffers& qb, const float* from, const float* to,
               const int* rayWorld, int n, int group, int mask, jbgpu_ray_hit* hits, int sms, cudaStream_t s) {
    if (n <= 0) return JBGPU_OK;
    int rc;
    if (!grow_ray_buffers(qb, n)) return JBGPU_ERR_CUDA;
    cudaMemsetAsync(qb.slowCount, 0, sizeof(int), s);
    cudaMemsetAsync(qb.key, 0xff, sizeof(unsigned long long) * n, s);
    cudaMemsetAsync(qb.undecided, 0, sizeof(int) * n, s);
    DevWorld wq = w;
    wq.amin = qb.qmin;
    wq.amax = qb.qmax;
    Bvh tree = bb.bvh;
    tree.node = qb.node;
    if (!qb.replayAll) {
        k_ray_walk<true><<<gridn(n, RAY_THREADS), RAY_THREADS, 0, s>>>(w, wq, bb.sortedBody, tree, bb.wroot, bb.planeList,
                                                                        bb.planeStart, from, to, rayWorld, n, bb.nWorlds,
                                                                        group, mask, qb.rayCnt, nullptr, nullptr);
        note_launch();
        exclusive_scan(qb.rayCnt, qb.rayOff, qb.candTotal, n, qb.scanScratch, s);
        int total = 0;
        if ((rc = candidate_total(qb, n, s, total)) != JBGPU_OK) return rc;
        if (!grow_cand_buffers(qb, total)) return JBGPU_ERR_CUDA;
        if (total > 0) {
            RayCand* cand = (RayCand*)qb.cand;
            k_ray_walk<false><<<gridn(n, RAY_THREADS), RAY_THREADS, 0, s>>>(w, wq, bb.sortedBody, tree, bb.wroot,
                                                                             bb.planeList, bb.planeStart, from, to, rayWorld,
                                                                             n, bb.nWorlds, group, mask, nullptr, qb.rayOff,
                                                                             cand);
            note_launch();
            k_ray_cast<<<gridn(total, RAY_THREADS), RAY_THREADS, 0, s>>>(w, cand, total, from, to, qb.hitA, qb.hitB, qb.key);
            note_launch();
            k_ray_pick<<<gridn(total, 256), 256, 0, s>>>(cand, total, qb.hitA, qb.hitB, qb.key, from, to, qb.enterJ, hits);
            note_launch();
            k_ray_check<<<gridn(total, 256), 256, 0, s>>>(cand, total, qb.hitA, qb.hitB, qb.key, qb.enterJ, qb.undecided);
            note_launch();
        }
    }
    k_ray_finish<<<gridn(n, 256), 256, 0, s>>>(n, qb.key, qb.undecided, qb.replayAll, hits, qb.slow, qb.slowCount);
    note_launch();
    k_rays_slow<<<sms, SLOW_THREADS, 0, s>>>(w, wq, from, to, rayWorld, group, mask, hits, qb.slow, qb.slowCount);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? JBGPU_OK : JBGPU_ERR_CUDA;
}

// Candidates of a batch too small to fill the GPU with one walk per sweep: a thread per
// (sweep, body) runs the walk's leaf test (filter, grown aabb entered before min(1, exit)).
// Counts the candidates and appends the first cap of them (order is immaterial: the casts keep
// the smallest key).
__global__ void k_sweep_list(DevWorld w, DevWorld wq, const float* ofrom, const float* oto, const int* sweepWorld, int n,
                             int nWorlds, int group, int mask, const float4* gmin, const float4* gmax,
                             unsigned long long* counter, RayCand* cand, int cap) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= w.nBodies) return;
    const int lane = threadIdx.x & 31;
    const V amn = mk4(wq.amin[b]), amx = mk4(wq.amax[b]);
    const int bw = w.world[b];
    const bool filt = passes_filter(w, b, group, mask);
    for (int q = blockIdx.y; q < n; q += gridDim.y) {
        bool pass = false;
        float enter = 0.0f, exit;
        const int sw = sweepWorld ? sweepWorld[q] : 0;
        if (b == 0 && (sw < 0 || sw >= nWorlds)) atomicOr(&w.ctr[C_STATUS], ST_BAD_WORLD);
        if (filt && bw == sw) {
            const V f = mk(ofrom[3 * q], ofrom[3 * q + 1], ofrom[3 * q + 2]);
            const V t = mk(oto[3 * q], oto[3 * q + 1], oto[3 * q + 2]);
            pass = ray_aabb_parts(f, t, add(amn, mk4(gmin[q])), add(amx, mk4(gmax[q])), enter, exit) &&
                   enter <= jmin(1.0f, exit);
        }
        const unsigned act = __activemask();
        const unsigned m = __ballot_sync(act, pass);
        if (!m) continue;
        const int leader = __ffs(m) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(m));
        base = __shfl_sync(act, base, leader);
        if (!pass) continue;
        const unsigned long long idx = base + __popc(m & ((1u << lane) - 1u));
        if (idx < (unsigned long long)cap) {
            RayCand rc;
            rc.ray = q;
            rc.body = b;
            rc.enter = enter;
            rc.pad = 0;
            cand[idx] = rc;
        }
    }
}

// One thread per candidate (sweep, body) of the tree walk: a static plane flags the sweep, any
// other body runs GjkConvexCast and offers (fraction, body) to the sweep's smallest key.
__global__ void __launch_bounds__(RAY_THREADS) k_sweep_cast(DevWorld w, const RayCand* cand, int total, int shape,
                                                           const float* from, const float* to, float4* hitA, float4* hitB,
                                                           unsigned long long* key, int* planeHit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const RayCand c = cand[i];
    const int bs = w.shape[c.body];
    if (w.sh.type[bs] == SHAPE_PLANE) {
        atomicOr(planeHit + c.ray, 1);
        return;
    }
    const Xf fa = xf12(from + 12 * c.ray);
    const V ta = mk(to[12 * c.ray + 9], to[12 * c.ray + 10], to[12 * c.ray + 11]);
    const Xf tb = load_xf(w, c.body);
    if (w.sh.type[bs] == SHAPE_MESH) {   // objectQuerySingle's BvhTriangleMeshShape branch
        Xf rot;
        rot.b = mulMM(xf_inverse(tb).b, xf12(to + 12 * c.ray).b);   // the end rotation in the mesh's space
        rot.o = mk(0.0f, 0.0f, 0.0f);
        V cbmin, cbmax;
        shape_aabb(w.sh, shape, rot, cbmin, cbmax);
        float best = 1.0f;
        sweep_mesh(w.sh, bs, tb, shape_ref(w.sh, shape), fa, ta, cbmin, cbmax, [&](float f, V n, V p) {
            best = f;                        // ClosestConvexResultCallback.addSingleResult
            hitA[i] = f4(n, f);              // k_sweep_pick applies processTriangle's normalisation
            hitB[i] = f4(p, 0.0f);
            return true;
        });
        if (best < 1.0f) atomicMin(key + c.ray, hit_key(best, c.body, 0));
        return;
    }
    // objectQuerySingle's convex branch, or its compound branch over the children at the body's
    // transform times the child's (CollisionWorld.java:391-430, 491-510): the first smallest hit
    const bool compound = w.sh.type[bs] == SHAPE_COMPOUND;
    const int nc = compound ? w.sh.child_cnt[bs] : 1;
    float best = 1.0f;   // ClosestConvexResultCallback starts at closestHitFraction 1
    for (int k = 0; k < nc; k++) {
        const int cc = compound ? w.sh.child_off[bs] + k : 0;
        float f;
        V nrm, p;
        if (!gjk_convex_cast(shape_ref(w.sh, shape), fa, ta, shape_ref(w.sh, compound ? w.sh.child_shape[cc] : bs),
                             compound ? xf_mul(tb, child_xf(w.sh, cc)) : tb, f, nrm, p) ||
            !(len2(nrm) > 0.0001f) || !(f < best))
            continue;
        best = f;
        hitA[i] = f4(nrm, f);
        hitB[i] = f4(p, 0.0f);
    }
    if (best < 1.0f) atomicMin(key + c.ray, hit_key(best, c.body, 0));
}

// The candidate holding its sweep's smallest key writes the record (one body per key).
__global__ void k_sweep_pick(const RayCand* cand, int total, const float4* hitA, const float4* hitB,
                             const unsigned long long* key, jbgpu_ray_hit* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const RayCand c = cand[i];
    const unsigned long long k = key[c.ray];
    if (k == ~0ull || (int)((k >> 1) & 0x7fffffffu) != c.body) return;
    const float4 a = hitA[i], b = hitB[i];
    jbgpu_ray_hit o;
    o.body = c.body;
    o.fraction = a.w;
    const V nn = nor(mk4(a));
    o.normal[0] = nn.x; o.normal[1] = nn.y; o.normal[2] = nn.z;
    o.point[0] = b.x; o.point[1] = b.y; o.point[2] = b.z;
    out[c.ray] = o;
}

__global__ void k_sweep_finish(int n, const unsigned long long* key, const int* planeHit, jbgpu_ray_hit* out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    if (!planeHit[q] && key[q] != ~0ull) return;
    jbgpu_ray_hit o;
    o.body = planeHit[q] ? -2 : -1;
    o.fraction = 1.0f;
    o.normal[0] = o.normal[1] = o.normal[2] = 0.0f;
    o.point[0] = o.point[1] = o.point[2] = 0.0f;
    out[q] = o;
}

int query_sweeps(const DevWorld& w, const BroadphaseBuffers& bb, QueryBuffers& qb, int shape, const float* from,
                 const float* to, const int* sweepWorld, int n, int group, int mask, jbgpu_ray_hit* hits, int sms,
                 cudaStream_t s) {
    if (n <= 0) return JBGPU_OK;
    if (!grow_ray_buffers(qb, n)) return JBGPU_ERR_CUDA;
    if (n > qb.capSweeps) {
        void* old[] = {qb.sweepMin, qb.sweepMax, qb.sweepPlane, qb.sweepFrom, qb.sweepTo};
        for (void* p : old)
            if (p) cudaFree(p);
        qb.sweepMin = qb.sweepMax = nullptr;
        qb.sweepPlane = nullptr;
        qb.sweepFrom = qb.sweepTo = nullptr;
        const int c = n > 2 * qb.capSweeps ? n : 2 * qb.capSweeps;
        qb.capSweeps = 0;
        if (cudaMalloc((void**)&qb.sweepMin, sizeof(float4) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.sweepMax, sizeof(float4) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.sweepPlane, sizeof(int) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.sweepFrom, sizeof(float) * 3 * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&qb.sweepTo, sizeof(float) * 3 * (size_t)c) != cudaSuccess)
            return JBGPU_ERR_CUDA;
        qb.capSweeps = c;
    }
    cudaMemsetAsync(qb.key, 0xff, sizeof(unsigned long long) * n, s);
    cudaMemsetAsync(qb.sweepPlane, 0, sizeof(int) * n, s);
    DevWorld wq = w;
    wq.amin = qb.qmin;
    wq.amax = qb.qmax;
    Bvh tree = bb.bvh;
    tree.node = qb.node;
    k_sweep_prep<<<gridn(n, 128), 128, 0, s>>>(w, shape, from, to, n, qb.sweepMin, qb.sweepMax, qb.sweepFrom, qb.sweepTo);
    note_launch();
    // a walk per sweep once the batch fills the GPU, else the (sweep, body) grid
    const bool walk = (long long)n >= 8LL * sms * RAY_THREADS;
    const dim3 grid(gridn(w.nBodies, 128), n < 65535 ? n : 65535);
    if (walk) {
        k_ray_walk<true, true><<<gridn(n, RAY_THREADS), RAY_THREADS, 0, s>>>(
            w, wq, bb.sortedBody, tree, bb.wroot, bb.planeList, bb.planeStart, qb.sweepFrom, qb.sweepTo, sweepWorld, n,
            bb.nWorlds, group, mask, qb.rayCnt, nullptr, nullptr, qb.sweepMin, qb.sweepMax);
        note_launch();
        exclusive_scan(qb.rayCnt, qb.rayOff, qb.candTotal, n, qb.scanScratch, s);
    } else {   // appended straight into the candidate buffer; listed again only if it overflowed
        cudaMemsetAsync(qb.candTotal64, 0, sizeof(unsigned long long), s);
        k_sweep_list<<<grid, 128, 0, s>>>(w, wq, qb.sweepFrom, qb.sweepTo, sweepWorld, n, bb.nWorlds, group, mask,
                                          qb.sweepMin, qb.sweepMax, qb.candTotal64, (RayCand*)qb.cand, qb.capCand);
        note_launch();
    }
    int total = 0;
    if (walk) {
        const int rc = candidate_total(qb, n, s, total);
        if (rc != JBGPU_OK) return rc;
    } else {
        unsigned long long t64 = 0;
        if (cudaMemcpyAsync(&t64, qb.candTotal64, sizeof(t64), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return JBGPU_ERR_CUDA;
        if (t64 > (unsigned long long)INT_MAX) return JBGPU_ERR_CAPACITY;
        total = (int)t64;
    }
    const bool listed = !walk && total <= qb.capCand;
    if (!grow_cand_buffers(qb, total)) return JBGPU_ERR_CUDA;
    if (total > 0) {
        RayCand* cand = (RayCand*)qb.cand;
        if (!listed) {
            if (walk) {
                k_ray_walk<false, true><<<gridn(n, RAY_THREADS), RAY_THREADS, 0, s>>>(
                    w, wq, bb.sortedBody, tree, bb.wroot, bb.planeList, bb.planeStart, qb.sweepFrom, qb.sweepTo, sweepWorld,
                    n, bb.nWorlds, group, mask, nullptr, qb.rayOff, cand, qb.sweepMin, qb.sweepMax);
            } else {
                cudaMemsetAsync(qb.candTotal64, 0, sizeof(unsigned long long), s);
                k_sweep_list<<<grid, 128, 0, s>>>(w, wq, qb.sweepFrom, qb.sweepTo, sweepWorld, n, bb.nWorlds, group, mask,
                                                  qb.sweepMin, qb.sweepMax, qb.candTotal64, cand, total);
            }
            note_launch();
        }
        k_sweep_cast<<<gridn(total, RAY_THREADS), RAY_THREADS, 0, s>>>(w, cand, total, shape, from, to, qb.hitA, qb.hitB,
                                                                     qb.key, qb.sweepPlane);
        note_launch();
        k_sweep_pick<<<gridn(total, 256), 256, 0, s>>>(cand, total, qb.hitA, qb.hitB, qb.key, hits);
        note_launch();
    }
    k_sweep_finish<<<gridn(n, 256), 256, 0, s>>>(n, qb.key, qb.sweepPlane, hits);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? JBGPU_OK : JBGPU_ERR_CUDA;
}

// ---- CCD motion clamping ---------------------------------------------------------------------
// integrateTransforms (dynamics/DiscreteDynamicsWorld.java:679-739) for worlds where some body has
// a CCD motion threshold.  The reference moves bodies one after the other; a body whose predicted
// displacement squared exceeds ccdMotionThreshold^2 first sweeps a SphereShape of its
// ccdSweptSphereRadius along its predicted motion with convexSweepTest (CollisionWorld.java:
// 596-645), the objects seen where they are at that moment: bodies before it in the world's
// order already moved, the rest not.  Here every body's predicted transform is computed at once;
// a body that runs no sweep ends there.  The sweeping bodies are then taken in index order by
// one cooperative launch: all threads test every object of the world against the sweep (seeing
// the finished transform of objects before the body and the old one of the rest), the smallest
// accepted fraction is reduced, and one thread clamps the body before the next one is taken.

// Predicted transforms (RigidBody.predictIntegratedTransform), and which bodies sweep.
__global__ void k_ccd_predict(DevWorld w, float dt, float4* pred, int* flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) w.ctr[C_CCD_BEST] = (int)__float_as_uint(1.0f);
    if (i >= w.nBodies) return;
    w.hitf[i] = 1.0f;
    Xf t = load_xf(w, i);
    int f = 0;
    if (is_active_state(w.act[i]) && !is_static_or_kin(w.flags[i])) {
        const Xf p = integrate_transform(t, mk4(w.linvel[i]), mk4(w.angvel[i]), dt);
        const float thr = w.ccdThr[i];
        const float sq = __fmul_rn(thr, thr);                 // getCcdSquareMotionThreshold
        const float squareMotion = len2(sub(p.o, t.o));
        // only a convex body sweeps (integrateTransforms' isConvex test, DiscreteDynamicsWorld.java:703)
        f = sq != 0.0f && sq < squareMotion && shape_is_convex(w.sh.type[w.shape[i]]) ? 1 : 0;
        t = p;
    }
    pred[3 * i] = make_float4(t.b.r[0].x, t.b.r[0].y, t.b.r[0].z, t.o.x);
    pred[3 * i + 1] = make_float4(t.b.r[1].x, t.b.r[1].y, t.b.r[1].z, t.o.y);
    pred[3 * i + 2] = make_float4(t.b.r[2].x, t.b.r[2].y, t.b.r[2].z, t.o.z);
    flag[i] = f;
}

__global__ void k_ccd_list(int n, const int* flag, const int* pos, int* list) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) list[pos[i]] = i;
}

JBD Xf ld_pred(const float4* pred, int i) {
    const float4 a = __ldcg(&pred[3 * i]), b = __ldcg(&pred[3 * i + 1]), c = __ldcg(&pred[3 * i + 2]);
    Xf t;
    t.b.r[0] = mk(a.x, a.y, a.z);
    t.b.r[1] = mk(b.x, b.y, b.z);
    t.b.r[2] = mk(c.x, c.y, c.z);
    t.o = mk(a.w, b.w, c.w);
    return t;
}

// Does the sweeping body `me` skip object j because it already touches it?  The reference asks
// HashedOverlappingPairCache.findPair (collision/broadphase/HashedOverlappingPairCache.java:
// 231-265), whose swap of its arguments is broken (233-237): the pair is found only when `me`
// precedes j (key (me << 32) | j: j is the partner whether it is a body or a plane); found with a
// manifold that holds contact points, j is skipped (DiscreteDynamicsWorld.java:1180-1195).
// A pair with a compound body has a manifold per child combination (key_sub); the algorithm's
// getAllContactManifolds lists them all, and any with points counts.
JBD bool ccd_touching(const DevWorld& w, const DevPairs& P, int np, int me, int j) {
    if (me > j) return false;
    const int subs = w.hasCompound ? pair_subs(w.sh, w.shape[me], w.shape[j]) : 1;
    for (int sub = 0; sub < subs; sub++) {
        const uint64_t key = ((uint64_t)(unsigned)me << 32) | ((unsigned)sub << 24) | (unsigned)j;
        int lo = 0, hi = np - 1;
        while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
            const uint64_t k = P.keys[mid];
            if (k == key) {
                if (P.has[mid] && P.n[mid] > 0) return true;
                break;
            }
            if (k < key) lo = mid + 1;
            else hi = mid - 1;
        }
    }
    return false;
}

// The sweeps, in index order (ClosestNotMeConvexResultCallback, DiscreteDynamicsWorld.java:
// 1129-1198, over convexSweepTest and objectQuerySingle, CollisionWorld.java:391-490,596-645).
// An accepted hit: GjkConvexCast found one with |normal|^2 > 0.0001 and the normalised normal
// opposes the motion; the callback keeps the closest, so the answer is the smallest accepted
// fraction whatever the object order.  Body moved to its transform after dt * fraction when one
// was accepted above 0.0001.  Static planes the sweep reaches are flagged (the reference throws).
__global__ void __launch_bounds__(256) k_ccd_sweep(DevWorld w, DevPairs P, int nPairs, const int* cntp, float4* pred,
                                                   const int* list, float dt) {
    __shared__ float sBox[6];
    __shared__ unsigned sBest;
    unsigned barK = 0;
    const int nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int count = __ldcg(&w.ctr[C_CCD_N]);
    const int np = cntp ? min(nPairs, __ldcg(cntp)) : nPairs;
    for (int k = 0; k < count; k++) {
        const int me = list[k];
        const Xf from = load_xf(w, me);
        const Xf to = ld_pred(pred, me);
        const float r = w.ccdRad[me];
        if (threadIdx.x == 0) {
            V mn, mx;
            cast_box(from, to, [&](const Xf& x, V& a, V& b) {   // SphereShape.getAabb: centre -+ radius
                a = sub(x.o, mk(r, r, r));
                b = add(x.o, mk(r, r, r));
            }, mn, mx);
            sBox[0] = mn.x; sBox[1] = mn.y; sBox[2] = mn.z;
            sBox[3] = mx.x; sBox[4] = mx.y; sBox[5] = mx.z;
            sBest = __float_as_uint(1.0f);
        }
        __syncthreads();
        const V cmin = mk(sBox[0], sBox[1], sBox[2]), cmax = mk(sBox[3], sBox[4], sBox[5]);
        const V motion = sub(to.o, from.o);
        const int wi = w.world[me], gm = w.group[me], mm = w.mask[me];
        const bool resp = (w.flags[me] & CF_NO_CONTACT_RESPONSE) == 0;
        ShapeRef cast;
        cast.type = SHAPE_SPHERE;
        cast.margin = r;
        cast.dims = mk(r, r, r);
        cast.up = 1;
        cast.pts = nullptr;
        cast.npts = 0;
        for (int j = tid; j < w.nBodies; j += nth) {
            if (j == me || w.world[j] != wi) continue;
            if (((w.group[j] & mm) & 0xFFFF) == 0 || ((gm & w.mask[j]) & 0xFFFF) == 0) continue;
            if (resp && (w.flags[j] & CF_NO_CONTACT_RESPONSE) == 0 && ccd_touching(w, P, np, me, j)) continue;
            const Xf tj = j < me ? ld_pred(pred, j) : load_xf(w, j);
            V bmn, bmx;
            shape_aabb(w.sh, w.shape[j], tj, bmn, bmx);
            float enter, exit;
            if (!(ray_aabb_parts(from.o, to.o, add(bmn, cmin), add(bmx, cmax), enter, exit) && enter <= jmin(1.0f, exit)))
                continue;
            if (w.sh.type[w.shape[j]] == SHAPE_PLANE) {
                atomicOr(&w.ctr[C_STATUS], ST_CCD_PLANE);
                continue;
            }
            const int sj = w.shape[j];
            if (w.sh.type[sj] == SHAPE_MESH) {   // the mesh branch; the sphere's box is -r .. r at any rotation
                sweep_mesh(w.sh, sj, tj, cast, from, to.o, mk(-r, -r, -r), mk(r, r, r), [&](float f, V n, V) {
                    if (dot(nor(n), motion) >= -0.0f) return false;   // ClosestNotMeConvexResultCallback rejects
                    atomicMin(&sBest, __float_as_uint(f));
                    return true;
                });
                continue;
            }
            const bool compound = w.sh.type[sj] == SHAPE_COMPOUND;   // the compound branch: every child
            for (int k = 0, nc = compound ? w.sh.child_cnt[sj] : 1; k < nc; k++) {
                const int cc = compound ? w.sh.child_off[sj] + k : 0;
                float f;
                V n, p;
                if (!gjk_convex_cast(cast, from, to.o, shape_ref(w.sh, compound ? w.sh.child_shape[cc] : sj),
                                     compound ? xf_mul(tj, child_xf(w.sh, cc)) : tj, f, n, p))
                    continue;
                if (!(len2(n) > 0.0001f) || !(f < 1.0f)) continue;
                if (dot(nor(n), motion) >= -0.0f) continue;        // moving away from the contact normal
                atomicMin(&sBest, __float_as_uint(f));
            }
        }
        __syncthreads();
        if (threadIdx.x == 0 && sBest < __float_as_uint(1.0f)) atomicMin((unsigned*)&w.ctr[C_CCD_BEST], sBest);
        grid_barrier(w.ctr, nb, barK);
        if (tid == 0) {
            const float f = __uint_as_float((unsigned)__ldcg(&w.ctr[C_CCD_BEST]));
            if (f < 1.0f && f > 0.0001f) {
                const Xf p = integrate_transform(from, mk4(w.linvel[me]), mk4(w.angvel[me]), __fmul_rn(dt, f));
                w.hitf[me] = 0.0f;   // integrateTransforms: setHitFraction(0) after the clamp
                pred[3 * me] = make_float4(p.b.r[0].x, p.b.r[0].y, p.b.r[0].z, p.o.x);
                pred[3 * me + 1] = make_float4(p.b.r[1].x, p.b.r[1].y, p.b.r[1].z, p.o.y);
                pred[3 * me + 2] = make_float4(p.b.r[2].x, p.b.r[2].y, p.b.r[2].z, p.o.z);
            }
            w.ctr[C_CCD_BEST] = (int)__float_as_uint(1.0f);
        }
        grid_barrier(w.ctr, nb, barK);
    }
}

// RigidBody.proceedToTransform: the final transforms and world inverse inertia of moved bodies.
__global__ void k_ccd_commit(DevWorld w, const float4* pred) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    if (!is_active_state(w.act[i]) || is_static_or_kin(w.flags[i])) return;
    const Xf p = ld_pred(pred, i);
    store_xf(w, i, p);
    store_interpolation(w, i, p);
    M m1 = scaleM(p.b, mk4(w.iloc[i]));
    M iw = mulMM(m1, transpose(p.b));
    w.iw0[i] = f4(iw.r[0], 0.0f);
    w.iw1[i] = f4(iw.r[1], 0.0f);
    w.iw2[i] = f4(iw.r[2], 0.0f);
}

int ccd_reserve(CcdBuffers& cb, int n, int sms) {
    if (n > cb.cap) {
        void* old[] = {cb.pred, cb.flag, cb.pos, cb.list, cb.scanScratch};
        for (void* p : old)
            if (p) cudaFree(p);
        cb.pred = nullptr;
        cb.flag = cb.pos = cb.list = nullptr;
        cb.scanScratch = nullptr;
        const int c = n > 2 * cb.cap ? n : 2 * cb.cap;
        cb.cap = 0;
        if (cudaMalloc((void**)&cb.pred, sizeof(float4) * 3 * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&cb.flag, sizeof(int) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&cb.pos, sizeof(int) * (size_t)c) != cudaSuccess ||
            cudaMalloc((void**)&cb.list, sizeof(int) * (size_t)c) != cudaSuccess ||
            cudaMalloc(&cb.scanScratch, scan_scratch_bytes(c)) != cudaSuccess)
            return JBGPU_ERR_CUDA;
        cb.cap = c;
    }
    if (!cb.grid) {
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ccd_sweep, 256, 0) != cudaSuccess || per < 1)
            return JBGPU_ERR_CUDA;
        cb.grid = sms * (per < 2 ? per : 2);
    }
    return JBGPU_OK;
}

int ccd_integrate(const DevWorld& w, const DevPairs& P, int nPairs, const int* cntp, CcdBuffers& cb, float dt, int sms,
                  cudaStream_t s) {
    const int n = w.nBodies;
    if (n <= 0) return JBGPU_OK;
    if (n > cb.cap || !cb.grid) {
        const int rc = ccd_reserve(cb, n, sms);
        if (rc) return rc;
    }
    k_ccd_predict<<<gridn(n, 256), 256, 0, s>>>(w, dt, cb.pred, cb.flag); note_launch();
    exclusive_scan(cb.flag, cb.pos, w.ctr + C_CCD_N, n, cb.scanScratch, s);
    k_ccd_list<<<gridn(n, 256), 256, 0, s>>>(n, cb.flag, cb.pos, cb.list); note_launch();
    cudaMemsetAsync(w.ctr + C_BAR_COUNT, 0, sizeof(int), s);
    {
        DevWorld wc = w;
        DevPairs pc = P;
        int npc = nPairs;
        const int* cc = cntp;
        float4* pr = cb.pred;
        const int* li = cb.list;
        float dtc = dt;
        void* args[] = {&wc, &pc, &npc, &cc, &pr, &li, &dtc};
        cudaLaunchCooperativeKernel((void*)k_ccd_sweep, cb.grid, 256, args, 0, s); note_launch();
    }
    k_ccd_commit<<<gridn(n, 256), 256, 0, s>>>(w, cb.pred); note_launch();
    return cudaGetLastError() == cudaSuccess ? JBGPU_OK : JBGPU_ERR_CUDA;
}

void ccd_free(CcdBuffers& cb) {
    void* ps[] = {cb.pred, cb.flag, cb.pos, cb.list, cb.scanScratch};
    for (void* p : ps)
        if (p) cudaFree(p);
    cb = CcdBuffers();
}

void query_free(QueryBuffers& qb) {
    void* ps[] = {qb.qmin, qb.qmax, qb.node, qb.visit, qb.slow, qb.slowCount, qb.from, qb.to, qb.rayWorld, qb.hits,
                  qb.rayCnt, qb.rayOff, qb.candTotal, qb.candTotal64, qb.key, qb.enterJ, qb.undecided, qb.scanScratch, qb.cand, qb.hitA,
                  qb.hitB, qb.sweepMin, qb.sweepMax, qb.sweepPlane, qb.sweepFrom, qb.sweepTo};
    for (void* p : ps)
        if (p) cudaFree(p);
    qb = QueryBuffers();
}

}  // namespace jbg
