// ORACLE (test infrastructure only): collision shapes on the reference's hot path.
// Citations relative to src/com/bulletphysics/.
#include "jb_world.h"

namespace jb {

float Shape::getMargin() const {
    if (type == SPHERE) return implicitDims.x * localScaling.x;   // SphereShape.getMargin -> getRadius (SphereShape.java:84-97)
    return collisionMargin;                                       // ConvexInternalShape.getMargin
}

// BoxShape(Vector3 boxHalfExtents): implicitShapeDimensions = halfExtents*scaling - margin (BoxShape.java:46-50)
Shape make_box(V3 he) {
    Shape s;
    s.type = BOX;
    V3 m = v3(s.collisionMargin, s.collisionMargin, s.collisionMargin);
    s.implicitDims = sub(mulc(he, s.localScaling), m);
    return s;
}

// SphereShape(radius) (SphereShape.java:38-41)
Shape make_sphere(float r) {
    Shape s;
    s.type = SPHERE;
    s.implicitDims.x = r;
    s.collisionMargin = r;
    return s;
}

// CapsuleShape(radius, height): up axis y, implicit dims (r, 0.5*height, r) (CapsuleShape.java:55-58)
Shape make_capsule(float r, float height) {
    Shape s;
    s.type = CAPSULE;
    s.upAxis = 1;
    s.implicitDims = v3(r, 0.5f * height, r);
    return s;
}

// PolyhedralConvexShape.recalcLocalAabb via ConvexHullShape.batchedUnitVectorGetSupportingVertexWithoutMargin
// (PolyhedralConvexShape.java:177-201, ConvexHullShape.java:104-139)
static void hull_recalc_local_aabb(Shape& s) {
    static const V3 dirs[6] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
    V3 sup[6];
    float wc[6];
    for (int j = 0; j < 6; j++) { wc[j] = -1e30f; sup[j] = v3(0, 0, 0); }
    for (size_t i = 0; i < s.points.size(); i++) {
        V3 vtx = mulc(s.points[i], s.localScaling);
        for (int j = 0; j < 6; j++) {
            float nd = dot(dirs[j], vtx);
            if (nd > wc[j]) { sup[j] = vtx; wc[j] = nd; }
        }
    }
    for (int i = 0; i < 3; i++) {
        set_coord(s.localAabbMax, i, coord(sup[i], i) + s.collisionMargin);
        set_coord(s.localAabbMin, i, coord(sup[i + 3], i) - s.collisionMargin);
    }
}

Shape make_hull(const float* pts, int n) {
    Shape s;
    s.type = CONVEX_HULL;
    for (int i = 0; i < n; i++) s.points.push_back(v3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
    hull_recalc_local_aabb(s);
    return s;
}

// StaticPlaneShape(normal, constant): normal.nor() (StaticPlaneShape.java:45-48)
Shape make_plane(V3 n, float c) {
    Shape s;
    s.type = STATIC_PLANE;
    s.planeNormal = nor(n);
    s.planeConstant = c;
    s.localScaling = v3(0, 0, 0);
    return s;
}

// AabbUtil2.transformAabb(halfExtents, margin, t) (linearmath/AabbUtil2.java:133-163)
static void transform_aabb_he(V3 he, float margin, const Xf& t, V3& mn, V3& mx) {
    V3 hem = v3(he.x + margin, he.y + margin, he.z + margin);
    M3 ab = absM(t.b);
    V3 c = t.o;
    V3 e = v3(dot(row(ab, 0), hem), dot(row(ab, 1), hem), dot(row(ab, 2), hem));
    mn = sub(c, e);
    mx = add(c, e);
}

// AabbUtil2.transformAabb(localMin, localMax, margin, t) (linearmath/AabbUtil2.java:165-209)
static void transform_aabb_mm(V3 lmin, V3 lmax, float margin, const Xf& t, V3& mn, V3& mx) {
    V3 lhe = scl(sub(lmax, lmin), 0.5f);
    lhe.x += margin; lhe.y += margin; lhe.z += margin;
    V3 lc = scl(add(lmax, lmin), 0.5f);
    M3 ab = absM(t.b);
    V3 c = xf_apply(t, lc);
    V3 e = v3(dot(row(ab, 0), lhe), dot(row(ab, 1), lhe), dot(row(ab, 2), lhe));
    mn = sub(c, e);
    mx = add(c, e);
}

void shape_aabb(const Shape& s, const Xf& t, V3& mn, V3& mx) {
    switch (s.type) {
    case BOX:      // BoxShape.getAabb (BoxShape.java:146-151)
        transform_aabb_he(s.implicitDims, s.getMargin(), t, mn, mx);
        break;
    case SPHERE: { // SphereShape.getAabb (SphereShape.java:56-65)
        float m = s.getMargin();
        V3 e = v3(m, m, m);
        mn = sub(t.o, e);
        mx = add(t.o, e);
        break;
    }
    case CAPSULE: { // CapsuleShape.getAabb (CapsuleShape.java:160-190)
        float r = s.capsuleRadius();
        V3 he = v3(r, r, r);
        set_coord(he, s.upAxis, r + s.capsuleHalfHeight());
        float m = s.getMargin();
        he.x += m; he.y += m; he.z += m;
        M3 ab = absM(t.b);
        V3 e = v3(dot(row(ab, 0), he), dot(row(ab, 1), he), dot(row(ab, 2), he));
        mn = sub(t.o, e);
        mx = add(t.o, e);
        break;
    }
    case CONVEX_HULL: // PolyhedralConvexShape.getAabb (PolyhedralConvexShape.java:163-171)
        transform_aabb_mm(s.localAabbMin, s.localAabbMax, s.getMargin(), t, mn, mx);
        break;
    default:          // StaticPlaneShape.getAabb (StaticPlaneShape.java:124-128)
        mn = v3(-1e30f, -1e30f, -1e30f);
        mx = v3(1e30f, 1e30f, 1e30f);
        break;
    }
}

static inline float fsel(float a, float b, float c) { return a >= 0 ? b : c; }  // ScalarUtil.fsel

static V3 normalize_dir(V3 vec) {   // shared prologue of the polyhedral/capsule support maps
    float lenSqr = len2(vec);
    if (lenSqr < 0.0001f) return v3(1, 0, 0);
    float rlen = 1.0f / jsqrt(lenSqr);
    return scl(vec, rlen);
}

V3 support_without_margin(const Shape& s, V3 vec) {
    switch (s.type) {
    case BOX: {   // BoxShape.localGetSupportingVertexWithoutMargin (BoxShape.java:86-97)
        V3 he = s.implicitDims;
        return v3(fsel(vec.x, he.x, -he.x), fsel(vec.y, he.y, -he.y), fsel(vec.z, he.z, -he.z));
    }
    case SPHERE:  // SphereShape.localGetSupportingVertexWithoutMargin (SphereShape.java:43-47)
        return v3(0, 0, 0);
    case CAPSULE: { // CapsuleShape.localGetSupportingVertexWithoutMargin (CapsuleShape.java:59-117)
        V3 sup = v3(0, 0, 0);
        float maxDot = -1e30f;
        V3 v = normalize_dir(vec);
        float radius = s.capsuleRadius();
        for (int k = 0; k < 2; k++) {
            V3 pos = v3(0, 0, 0);
            set_coord(pos, s.upAxis, k == 0 ? s.capsuleHalfHeight() : -s.capsuleHalfHeight());
            V3 tmp1 = scl(mulc(v, s.localScaling), radius);
            V3 tmp2 = scl(v, s.getMargin());
            V3 vtx = sub(add(pos, tmp1), tmp2);
            float nd = dot(v, vtx);
            if (nd > maxDot) { maxDot = nd; sup = vtx; }
        }
        return sup;
    }
    case CONVEX_HULL: { // ConvexHullShape.localGetSupportingVertexWithoutMargin (ConvexHullShape.java:74-102)
        V3 sup = v3(0, 0, 0);
        float maxDot = -1e30f;
        V3 v = normalize_dir(vec);
        for (size_t i = 0; i < s.points.size(); i++) {
            V3 vtx = mulc(s.points[i], s.localScaling);
            float nd = dot(v, vtx);
            if (nd > maxDot) { maxDot = nd; sup = vtx; }
        }
        return sup;
    }
    default:
        return v3(0, 0, 0);
    }
}

V3 support_with_margin(const Shape& s, V3 vec) {
    if (s.type == BOX) {   // BoxShape.localGetSupportingVertex (BoxShape.java:72-84)
        V3 he = s.implicitDims;
        float m = s.getMargin();
        he.x += m; he.y += m; he.z += m;
        return v3(fsel(vec.x, he.x, -he.x), fsel(vec.y, he.y, -he.y), fsel(vec.z, he.z, -he.z));
    }
    // ConvexInternalShape.localGetSupportingVertex (ConvexInternalShape.java:84-100),
    // identical in ConvexHullShape.localGetSupportingVertex (ConvexHullShape.java:141-157)
    V3 sup = support_without_margin(s, vec);
    if (s.getMargin() != 0.0f) {
        V3 vn = vec;
        if (len2(vn) < (FLT_EPS * FLT_EPS)) vn = v3(-1, -1, -1);
        vn = nor(vn);
        vn = scl(vn, s.getMargin());
        sup = add(sup, vn);
    }
    return sup;
}

V3 shape_local_inertia(const Shape& s, float mass) {
    switch (s.type) {
    case BOX: {   // BoxShape.calculateLocalInertia (BoxShape.java:153-167)
        float m = s.getMargin();
        V3 he = v3(s.implicitDims.x + m, s.implicitDims.y + m, s.implicitDims.z + m);
        float lx = 2.0f * he.x, ly = 2.0f * he.y, lz = 2.0f * he.z;
        return v3(mass / 12.0f * (ly * ly + lz * lz), mass / 12.0f * (lx * lx + lz * lz), mass / 12.0f * (lx * lx + ly * ly));
    }
    case SPHERE: { // SphereShape.calculateLocalInertia (SphereShape.java:72-76)
        float e = 0.4f * mass * s.getMargin() * s.getMargin();
        return v3(e, e, e);
    }
    case CAPSULE: { // CapsuleShape.calculateLocalInertia (CapsuleShape.java:125-153)
        float r = s.capsuleRadius();
        V3 he = v3(r, r, r);
        set_coord(he, s.upAxis, r + s.capsuleHalfHeight());
        float margin = 0.04f;
        float lx = 2.0f * (he.x + margin), ly = 2.0f * (he.y + margin), lz = 2.0f * (he.z + margin);
        float x2 = lx * lx, y2 = ly * ly, z2 = lz * lz;
        float sm = mass * 0.08333333f;
        return v3(sm * (y2 + z2), sm * (x2 + z2), sm * (x2 + y2));
    }
    case CONVEX_HULL: { // PolyhedralConvexShape.calculateLocalInertia (PolyhedralConvexShape.java:133-159)
        float margin = s.getMargin();
        V3 mn, mx;
        shape_aabb(s, xf_identity(), mn, mx);
        V3 he = scl(sub(mx, mn), 0.5f);
        float lx = 2.0f * (he.x + margin), ly = 2.0f * (he.y + margin), lz = 2.0f * (he.z + margin);
        float x2 = lx * lx, y2 = ly * ly, z2 = lz * lz;
        float sm = mass * 0.08333333f;
        return scl(v3(y2 + z2, x2 + z2, x2 + y2), sm);
    }
    default:        // StaticPlaneShape.calculateLocalInertia (StaticPlaneShape.java:151-154)
        return v3(0, 0, 0);
    }
}

}  // namespace jb
