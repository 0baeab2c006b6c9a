// Shape queries on the device: aabb and support maps of the shapes on the path
// (collision/shapes/{BoxShape,SphereShape,CapsuleShape,ConvexHullShape,StaticPlaneShape,
// TriangleShape,CompoundShape,TriangleMeshShape}.java).
// Local scaling is always (1,1,1) here, so the reference's multiplications by the scaling
// vector are exact identities and are omitted.
#pragma once
#include "jbgpu_internal.cuh"

namespace jbg {
using namespace jbd;

// AabbUtil2.transformAabb(halfExtents, margin, t) (linearmath/AabbUtil2.java:133-163)
JBD void transform_aabb_he(V he, float margin, const Xf& t, V& mn, V& mx) {
    V hem = mk(__fadd_rn(he.x, margin), __fadd_rn(he.y, margin), __fadd_rn(he.z, margin));
    M ab = absM(t.b);
    V e = mk(dot(ab.r[0], hem), dot(ab.r[1], hem), dot(ab.r[2], hem));
    mn = sub(t.o, e);
    mx = add(t.o, e);
}

JBD void shape_aabb(const DevShapes& sh, int s, const Xf& t, V& mn, V& mx) {
    int type = sh.type[s];
    float m = sh.margin[s];
    float4 d = sh.dims[s];
    if (type == SHAPE_BOX) {                  // BoxShape.getAabb
        transform_aabb_he(mk(d.x, d.y, d.z), m, t, mn, mx);
    } else if (type == SHAPE_SPHERE) {        // SphereShape.getAabb
        V e = mk(m, m, m);
        mn = sub(t.o, e);
        mx = add(t.o, e);
    } else if (type == SHAPE_CAPSULE) {       // CapsuleShape.getAabb
        int up = (int)d.w;
        V dv = mk(d.x, d.y, d.z);
        float r = coord(dv, (up + 2) % 3);
        V he = mk(r, r, r);
        set_coord(he, up, __fadd_rn(r, coord(dv, up)));
        he = mk(__fadd_rn(he.x, m), __fadd_rn(he.y, m), __fadd_rn(he.z, m));
        M ab = absM(t.b);
        V e = mk(dot(ab.r[0], he), dot(ab.r[1], he), dot(ab.r[2], he));
        mn = sub(t.o, e);
        mx = add(t.o, e);
    } else if (type == SHAPE_HULL || type == SHAPE_COMPOUND) {
        // PolyhedralConvexShape.getAabb -> transformAabb(min,max,margin,t); CompoundShape.getAabb
        // (CompoundShape.java:126-171) is the same arithmetic over its children's union
        V lmin = mk4(sh.laabb_min[s]), lmax = mk4(sh.laabb_max[s]);
        V lhe = scl(sub(lmax, lmin), 0.5f);
        lhe = mk(__fadd_rn(lhe.x, m), __fadd_rn(lhe.y, m), __fadd_rn(lhe.z, m));
        V lc = scl(add(lmax, lmin), 0.5f);
        M ab = absM(t.b);
        V c = xf_apply(t, lc);
        V e = mk(dot(ab.r[0], lhe), dot(ab.r[1], lhe), dot(ab.r[2], lhe));
        mn = sub(c, e);
        mx = add(c, e);
    } else if (type == SHAPE_MESH) {          // TriangleMeshShape.getAabb: the margin widens the extent
        V lmin = mk4(sh.laabb_min[s]), lmax = mk4(sh.laabb_max[s]);
        V lhe = scl(sub(lmax, lmin), 0.5f);
        V lc = scl(add(lmax, lmin), 0.5f);
        M ab = absM(t.b);
        V c = xf_apply(t, lc);
        V e = mk(dot(ab.r[0], lhe), dot(ab.r[1], lhe), dot(ab.r[2], lhe));
        e = mk(__fadd_rn(e.x, m), __fadd_rn(e.y, m), __fadd_rn(e.z, m));
        mn = sub(c, e);
        mx = add(c, e);
    } else {                                  // StaticPlaneShape.getAabb
        mn = mk(-1e30f, -1e30f, -1e30f);
        mx = mk(1e30f, 1e30f, 1e30f);
    }
}

JBD float fsel(float a, float b, float c) { return a >= 0 ? b : c; }

JBD V normalize_dir(V v) {
    float l2 = len2(v);
    if (l2 < 0.0001f) return mk(1.0f, 0.0f, 0.0f);
    return scl(v, jdiv(1.0f, jsqrt(l2)));
}

// Shape parameters gathered once per query.
struct ShapeRef {
    int type;
    float margin;
    V dims;
    int up;
    const float4* pts;
    int npts;
};
// A mesh triangle as the TriangleShape ConvexTriangleCallback collides (margin: the mesh's).
JBD ShapeRef triangle_ref(const DevShapes& sh, int meshShape, int tri) {
    ShapeRef r;
    r.type = SHAPE_TRIANGLE;
    r.margin = sh.margin[meshShape];
    r.dims = mk(0.0f, 0.0f, 0.0f);
    r.up = 1;
    r.pts = sh.mesh_tris + (size_t)3 * (sh.mesh_tri_off[meshShape] + tri);
    r.npts = 3;
    return r;
}
JBD ShapeRef shape_ref(const DevShapes& sh, int s) {
    ShapeRef r;
    r.type = sh.type[s];
    r.margin = sh.margin[s];
    float4 d = sh.dims[s];
    r.dims = mk(d.x, d.y, d.z);
    r.up = (int)d.w;
    r.pts = sh.hull_pts + sh.hull_off[s];
    r.npts = sh.hull_cnt[s];
    return r;
}

JBD V support_without_margin(const ShapeRef& s, V vec) {
    if (s.type == SHAPE_BOX) {                // BoxShape.localGetSupportingVertexWithoutMargin
        V he = s.dims;
        return mk(fsel(vec.x, he.x, -he.x), fsel(vec.y, he.y, -he.y), fsel(vec.z, he.z, -he.z));
    }
    if (s.type == SHAPE_SPHERE) return mk(0.0f, 0.0f, 0.0f);
    if (s.type == SHAPE_CAPSULE) {            // CapsuleShape.localGetSupportingVertexWithoutMargin
        V v = normalize_dir(vec);
        float radius = coord(s.dims, (s.up + 2) % 3);
        float hh = coord(s.dims, s.up);
        V sup = mk(0.0f, 0.0f, 0.0f);
        float maxDot = -1e30f;
        V t1 = scl(v, radius);
        V t2 = scl(v, s.margin);
        for (int k = 0; k < 2; k++) {
            V pos = mk(0.0f, 0.0f, 0.0f);
            set_coord(pos, s.up, k == 0 ? hh : -hh);
            V vtx = sub(add(pos, t1), t2);
            float nd = dot(v, vtx);
            if (nd > maxDot) { maxDot = nd; sup = vtx; }
        }
        return sup;
    }
    if (s.type == SHAPE_TRIANGLE) {           // TriangleShape.localGetSupportingVertexWithoutMargin with
        float mv = -1e30f;                    // VectorUtil.maxAxis (no normalisation; vertex 0 where
        V sup = mk4(s.pts[0]);                // the reference would index -1)
        for (int i = 0; i < 3; i++) {
            V vtx = mk4(s.pts[i]);
            float nd = dot(vec, vtx);
            if (nd > mv) { mv = nd; sup = vtx; }
        }
        return sup;
    }
    if (s.type == SHAPE_HULL) {               // ConvexHullShape.localGetSupportingVertexWithoutMargin
        V v = normalize_dir(vec);
        V sup = mk(0.0f, 0.0f, 0.0f);
        float maxDot = -1e30f;
        for (int i = 0; i < s.npts; i++) {
            float4 p = s.pts[i];
            V vtx = mk(p.x, p.y, p.z);
            float nd = dot(v, vtx);
            if (nd > maxDot) { maxDot = nd; sup = vtx; }
        }
        return sup;
    }
    return mk(0.0f, 0.0f, 0.0f);
}

JBD V support_with_margin(const ShapeRef& s, V vec) {
    if (s.type == SHAPE_BOX) {                // BoxShape.localGetSupportingVertex
        float m = s.margin;
        V he = mk(__fadd_rn(s.dims.x, m), __fadd_rn(s.dims.y, m), __fadd_rn(s.dims.z, m));
        return mk(fsel(vec.x, he.x, -he.x), fsel(vec.y, he.y, -he.y), fsel(vec.z, he.z, -he.z));
    }
    // ConvexInternalShape.localGetSupportingVertex / ConvexHullShape.localGetSupportingVertex
    V sup = support_without_margin(s, vec);
    if (s.margin != 0.0f) {
        V vn = vec;
        if (len2(vn) < __fmul_rn(FLT_EPS, FLT_EPS)) vn = mk(-1.0f, -1.0f, -1.0f);
        vn = nor(vn);
        vn = scl(vn, s.margin);
        sup = add(sup, vn);
    }
    return sup;
}

}  // namespace jbg
