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
    case COMPOUND:    // CompoundShape.getAabb (CompoundShape.java:126-171): the margin widens the half extents
        transform_aabb_mm(s.localAabbMin, s.localAabbMax, s.getMargin(), t, mn, mx);
        break;
    case TRIANGLE_MESH: { // TriangleMeshShape.getAabb (TriangleMeshShape.java:111-146): the margin widens the extent
        V3 lhe = scl(sub(s.localAabbMax, s.localAabbMin), 0.5f);
        V3 lc = scl(add(s.localAabbMax, s.localAabbMin), 0.5f);
        M3 ab = absM(t.b);
        V3 c = xf_apply(t, lc);
        V3 e = v3(dot(row(ab, 0), lhe), dot(row(ab, 1), lhe), dot(row(ab, 2), lhe));
        float m = s.getMargin();
        e.x += m; e.y += m; e.z += m;
        mn = sub(c, e);
        mx = add(c, e);
        break;
    }
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
    case TRIANGLE: { // TriangleShape.localGetSupportingVertexWithoutMargin (TriangleShape.java:95-103) with
                     // VectorUtil.maxAxis (linearmath/VectorUtil.java:41-58); the reference would index -1 when
                     // no dot exceeds -1e30, vertex 0 is taken here
        float d[3] = {dot(vec, s.tri[0]), dot(vec, s.tri[1]), dot(vec, s.tri[2])};
        int mi = 0;
        float mv = -1e30f;
        for (int k = 0; k < 3; k++) if (d[k] > mv) { mi = k; mv = d[k]; }
        return s.tri[mi];
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
    case COMPOUND: { // CompoundShape.calculateLocalInertia (CompoundShape.java:222-243): the aabb's box
        V3 mn, mx;
        shape_aabb(s, xf_identity(), mn, mx);
        V3 he = scl(sub(mx, mn), 0.5f);
        float lx = 2.0f * he.x, ly = 2.0f * he.y, lz = 2.0f * he.z;
        return v3((mass / 12.0f) * (ly * ly + lz * lz), (mass / 12.0f) * (lx * lx + lz * lz), (mass / 12.0f) * (lx * lx + ly * ly));
    }
    default:        // StaticPlaneShape / TriangleMeshShape.calculateLocalInertia (StaticPlaneShape.java:151-154,
                    // TriangleMeshShape.java:155-160): zero
        return v3(0, 0, 0);
    }
}

// ---- CompoundShape ---------------------------------------------------------------------
// CompoundShape.addChildShape (CompoundShape.java:59-91): the local aabb is the union of the
// children's aabbs at their transforms (VectorUtil.setMin / setMax = Math.min / max).
Shape make_compound(const std::vector<Shape>& children, const std::vector<Xf>& xf, float margin) {
    Shape s;
    s.type = COMPOUND;
    s.collisionMargin = 0.0f;
    s.localAabbMin = v3(1e30f, 1e30f, 1e30f);
    s.localAabbMax = v3(-1e30f, -1e30f, -1e30f);
    for (size_t i = 0; i < children.size(); i++) {
        V3 mn, mx;
        shape_aabb(children[i], xf[i], mn, mx);
        s.localAabbMin = v3(jmin(s.localAabbMin.x, mn.x), jmin(s.localAabbMin.y, mn.y), jmin(s.localAabbMin.z, mn.z));
        s.localAabbMax = v3(jmax(s.localAabbMax.x, mx.x), jmax(s.localAabbMax.y, mx.y), jmax(s.localAabbMax.z, mx.z));
        s.children.push_back(children[i]);
        s.childXf.push_back(xf[i]);
    }
    s.collisionMargin = margin;   // CompoundShape.setMargin; getAabb reads it, the local aabb does not
    return s;
}

// ---- BvhTriangleMeshShape / OptimizedBvh (quantized) ----------------------------------
namespace {
struct BvhBuild {
    QuantizedBvh& t;
    std::vector<uint16_t> leafQ;      // quantizedLeafNodes: 6 per leaf
    std::vector<int> leafTri;
    // OptimizedBvh.quantizeWithClamp (OptimizedBvh.java:1038-1056)
    void quantize(V3 p, uint16_t out[3]) const {
        V3 c = v3(jmax(p.x, t.bvhAabbMin.x), jmax(p.y, t.bvhAabbMin.y), jmax(p.z, t.bvhAabbMin.z));
        c = v3(jmin(c.x, t.bvhAabbMax.x), jmin(c.y, t.bvhAabbMax.y), jmin(c.z, t.bvhAabbMax.z));
        V3 v = mulc(sub(c, t.bvhAabbMin), t.bvhQuantization);
        out[0] = (uint16_t)((int)(v.x + 0.5f) & 0xFFFF);
        out[1] = (uint16_t)((int)(v.y + 0.5f) & 0xFFFF);
        out[2] = (uint16_t)((int)(v.z + 0.5f) & 0xFFFF);
    }
    // OptimizedBvh.unQuantize (OptimizedBvh.java:1058-1068)
    V3 unquantize(const uint16_t* q) const {
        V3 v = v3((float)q[0] / t.bvhQuantization.x, (float)q[1] / t.bvhQuantization.y, (float)q[2] / t.bvhQuantization.z);
        return add(v, t.bvhAabbMin);
    }
    V3 leafMin(int i) const { return unquantize(&leafQ[6 * i]); }     // getAabbMin (java:106-115)
    V3 leafMax(int i) const { return unquantize(&leafQ[6 * i + 3]); }
    V3 centre(int i) const { return scl(add(leafMax(i), leafMin(i)), 0.5f); }
    // OptimizedBvh.calcSplittingAxis (java:676-707)
    int splitAxis(int a, int b) const {
        int n = b - a;
        V3 means = v3(0, 0, 0), var = v3(0, 0, 0);
        for (int i = a; i < b; i++) means = add(means, centre(i));
        means = scl(means, 1.0f / (float)n);
        for (int i = a; i < b; i++) {
            V3 d = sub(centre(i), means);
            var = add(var, mulc(d, d));
        }
        var = scl(var, 1.0f / ((float)n - 1.0f));
        int mi = -1;
        float mv = -1e30f;
        for (int k = 0; k < 3; k++) if (coord(var, k) > mv) { mi = k; mv = coord(var, k); }
        return mi < 0 ? 2 : mi;   // VectorUtil.getCoord's default branch reads z
    }
    void swapLeaves(int i, int j) {
        for (int k = 0; k < 6; k++) std::swap(leafQ[6 * i + k], leafQ[6 * j + k]);
        std::swap(leafTri[i], leafTri[j]);
    }
    // OptimizedBvh.sortAndCalcSplittingIndex (java:622-674)
    int splitIndex(int a, int b, int axis) {
        int n = b - a, split = a;
        V3 means = v3(0, 0, 0);
        for (int i = a; i < b; i++) means = add(means, centre(i));
        means = scl(means, 1.0f / (float)n);
        float sv = coord(means, axis);
        for (int i = a; i < b; i++)
            if (coord(centre(i), axis) > sv) { swapLeaves(i, split); split++; }
        int rb = n / 3;
        if (split <= a + rb || split >= b - 1 - rb) split = a + (n >> 1);
        return split;
    }
    // OptimizedBvh.buildTree (java:480-561); the subtree headers only serve the cache-friendly
    // walk and are not built
    void build(int a, int b) {
        int n = b - a, cur = t.curNodeIndex;
        if (n == 1) {
            for (int k = 0; k < 6; k++) t.q[6 * cur + k] = leafQ[6 * a + k];
            t.escOrTri[cur] = leafTri[a];
            t.curNodeIndex++;
            return;
        }
        int axis = splitAxis(a, b);
        int split = splitIndex(a, b, axis);
        int node = t.curNodeIndex;
        quantize(v3(-1e30f, -1e30f, -1e30f), &t.q[6 * node + 3]);   // setInternalNodeAabbMax
        quantize(v3(1e30f, 1e30f, 1e30f), &t.q[6 * node]);          // setInternalNodeAabbMin
        for (int i = a; i < b; i++) {                                 // mergeInternalNodeAabb
            uint16_t qa[3], qb[3];
            quantize(leafMin(i), qa);
            quantize(leafMax(i), qb);
            for (int k = 0; k < 3; k++) {
                if (t.q[6 * node + k] > qa[k]) t.q[6 * node + k] = qa[k];
                if (t.q[6 * node + 3 + k] < qb[k]) t.q[6 * node + 3 + k] = qb[k];
            }
        }
        t.curNodeIndex++;
        build(a, split);
        build(split, b);
        t.escOrTri[node] = -(t.curNodeIndex - cur);                   // setInternalNodeEscapeIndex
    }
};
}  // namespace

Shape make_mesh(const float* vtx, int nv, const int* idx, int nt, float margin, V3 scaling) {
    Shape s;
    s.type = TRIANGLE_MESH;
    s.collisionMargin = 0.0f;   // ConcaveShape.collisionMargin
    // BvhTriangleMeshShape.setLocalScaling (java:195-212): the mesh interface's scaling is set,
    // and the tree rebuilt over the scaled triangles, only when the scaling differs from the
    // current (1, 1, 1) by a squared length above SIMD_EPSILON; the margin is still 0 then, so the
    // rebuilt tree's quantization bounds equal the brute-force box of the scaled vertices
    bool scaled = false;
    if (!(scaling.x == 0.0f && scaling.y == 0.0f && scaling.z == 0.0f)) {
        const V3 d = sub(v3(1.0f, 1.0f, 1.0f), scaling);
        scaled = len2(d) > 1.1920929e-7f;
    }
    auto md = std::make_shared<MeshData>();
    md->idx.assign(idx, idx + (size_t)3 * nt);
    md->numVertices = nv;
    md->scaling = scaling;
    md->scaled = scaled;
    md->tri.resize((size_t)3 * nt);
    for (int i = 0; i < nt; i++)   // VertexData.getTriangle (VertexData.java:50-55): vertex times scaling
        for (int k = 0; k < 3; k++) {
            int v = idx[3 * i + k];
            V3 p = v3(vtx[3 * v], vtx[3 * v + 1], vtx[3 * v + 2]);
            if (scaled) p = v3(p.x * scaling.x, p.y * scaling.y, p.z * scaling.z);
            md->tri[3 * i + k] = p;
        }
    (void)nv;
    // StridingMeshInterface.calculateAabbBruteForce (StridingMeshInterface.java:70-87)
    V3 amin = v3(1e30f, 1e30f, 1e30f), amax = v3(-1e30f, -1e30f, -1e30f);
    for (const V3& p : md->tri) {
        amin = v3(jmin(amin.x, p.x), jmin(amin.y, p.y), jmin(amin.z, p.z));
        amax = v3(jmax(amax.x, p.x), jmax(amax.y, p.y), jmax(amax.z, p.z));
    }
    // OptimizedBvh.build (java:283-342) with setQuantizationValues(aabbMin, aabbMax, 1) (java:128-144)
    QuantizedBvh& t = md->bvh;
    t.bvhAabbMin = sub(amin, v3(1, 1, 1));
    t.bvhAabbMax = add(amax, v3(1, 1, 1));
    V3 size = sub(t.bvhAabbMax, t.bvhAabbMin);
    t.bvhQuantization = v3(65535.0f / size.x, 65535.0f / size.y, 65535.0f / size.z);
    BvhBuild b{t, {}, {}};
    b.leafQ.resize((size_t)6 * nt);
    b.leafTri.resize(nt);
    for (int i = 0; i < nt; i++) {   // QuantizedNodeTriangleCallback.internalProcessTriangleIndex (java:240-280)
        V3 mn = v3(1e30f, 1e30f, 1e30f), mx = v3(-1e30f, -1e30f, -1e30f);
        for (int k = 0; k < 3; k++) {
            V3 p = md->tri[3 * i + k];
            mn = v3(jmin(mn.x, p.x), jmin(mn.y, p.y), jmin(mn.z, p.z));
            mx = v3(jmax(mx.x, p.x), jmax(mx.y, p.y), jmax(mx.z, p.z));
        }
        for (int k = 0; k < 3; k++)
            if (coord(mx, k) - coord(mn, k) < 0.002f) {
                set_coord(mx, k, coord(mx, k) + 0.001f);
                set_coord(mn, k, coord(mn, k) - 0.001f);
            }
        b.quantize(mn, &b.leafQ[6 * i]);
        b.quantize(mx, &b.leafQ[6 * i + 3]);
        b.leafTri[i] = (0 << 21) | i;
    }
    t.q.assign((size_t)12 * nt, 0);
    t.escOrTri.assign((size_t)2 * nt, 0);
    t.curNodeIndex = 0;
    b.build(0, nt);
    s.mesh = md;
    // TriangleMeshShape.recalcLocalAabb (TriangleMeshShape.java:79-95) with the support callback
    // over every triangle in walk order (java:206-227), collisionMargin 0 at that time
    for (int i = 0; i < 3; i++) {
        for (int sg = 0; sg < 2; sg++) {
            float best = -1e30f;
            V3 sup = v3(0, 0, 0);
            for (int node = 0; node < t.curNodeIndex; node++) {
                if (t.escOrTri[node] < 0) continue;
                int tri = t.escOrTri[node] & ((1 << 21) - 1);
                for (int k = 0; k < 3; k++) {
                    V3 p = md->tri[3 * tri + k];
                    V3 dir = v3(0, 0, 0);
                    set_coord(dir, i, sg == 0 ? 1.0f : -1.0f);
                    float d = dot(dir, p);
                    if (d > best) { best = d; sup = p; }
                }
            }
            if (sg == 0) set_coord(s.localAabbMax, i, coord(sup, i) + 0.0f);
            else set_coord(s.localAabbMin, i, coord(sup, i) - 0.0f);
        }
    }
    s.collisionMargin = margin;   // ConcaveShape.setMargin after construction
    return s;
}

// BvhTriangleMeshShape.refitTree (BvhTriangleMeshShape.java:172-178) after the mesh interface's
// vertices were replaced: OptimizedBvh.refit (OptimizedBvh.java:344-367) takes the quantization
// from the new brute-force box, and updateBvhNodes (java:411-470) requantizes the nodes from the
// last to the first - a leaf from its triangle's box (without the build's minimum extent), an
// internal node as the union of its two children's quantized boxes (the right child follows the
// left one's subtree); recalcLocalAabb then runs with the shape's current margin.
void mesh_refit(Shape& s, const float* vtx) {
    MeshData& md = const_cast<MeshData&>(*s.mesh);   // the world's own mesh (make_mesh made it)
    const int nt = (int)md.tri.size() / 3;
    for (int i = 0; i < nt; i++)
        for (int k = 0; k < 3; k++) {
            int v = md.idx[3 * i + k];
            V3 p = v3(vtx[3 * v], vtx[3 * v + 1], vtx[3 * v + 2]);
            if (md.scaled) p = v3(p.x * md.scaling.x, p.y * md.scaling.y, p.z * md.scaling.z);
            md.tri[3 * i + k] = p;
        }
    V3 amin = v3(1e30f, 1e30f, 1e30f), amax = v3(-1e30f, -1e30f, -1e30f);   // calculateAabbBruteForce
    for (const V3& p : md.tri) {
        amin = v3(jmin(amin.x, p.x), jmin(amin.y, p.y), jmin(amin.z, p.z));
        amax = v3(jmax(amax.x, p.x), jmax(amax.y, p.y), jmax(amax.z, p.z));
    }
    QuantizedBvh& t = md.bvh;
    t.bvhAabbMin = sub(amin, v3(1, 1, 1));   // setQuantizationValues, quantizationMargin 1
    t.bvhAabbMax = add(amax, v3(1, 1, 1));
    V3 size = sub(t.bvhAabbMax, t.bvhAabbMin);
    t.bvhQuantization = v3(65535.0f / size.x, 65535.0f / size.y, 65535.0f / size.z);
    BvhBuild b{t, {}, {}};
    for (int i = t.curNodeIndex - 1; i >= 0; i--) {
        if (t.escOrTri[i] >= 0) {
            const int tri = t.escOrTri[i] & ((1 << 21) - 1);
            V3 mn = v3(1e30f, 1e30f, 1e30f), mx = v3(-1e30f, -1e30f, -1e30f);
            for (int k = 0; k < 3; k++) {
                V3 p = md.tri[3 * tri + k];
                mn = v3(jmin(mn.x, p.x), jmin(mn.y, p.y), jmin(mn.z, p.z));
                mx = v3(jmax(mx.x, p.x), jmax(mx.y, p.y), jmax(mx.z, p.z));
            }
            b.quantize(mn, &t.q[6 * i]);
            b.quantize(mx, &t.q[6 * i + 3]);
        } else {
            const int l = i + 1;
            const int r = t.escOrTri[l] >= 0 ? i + 2 : i + 1 - t.escOrTri[l];
            for (int k = 0; k < 3; k++) {
                t.q[6 * i + k] = t.q[6 * l + k];
                if (t.q[6 * i + k] > t.q[6 * r + k]) t.q[6 * i + k] = t.q[6 * r + k];
                t.q[6 * i + 3 + k] = t.q[6 * l + 3 + k];
                if (t.q[6 * i + 3 + k] < t.q[6 * r + 3 + k]) t.q[6 * i + 3 + k] = t.q[6 * r + 3 + k];
            }
        }
    }
    const float m = s.collisionMargin;
    for (int i = 0; i < 3; i++) {
        for (int sg = 0; sg < 2; sg++) {
            float best = -1e30f;
            V3 sup = v3(0, 0, 0);
            for (int node = 0; node < t.curNodeIndex; node++) {
                if (t.escOrTri[node] < 0) continue;
                int tri = t.escOrTri[node] & ((1 << 21) - 1);
                for (int k = 0; k < 3; k++) {
                    V3 p = md.tri[3 * tri + k];
                    V3 dir = v3(0, 0, 0);
                    set_coord(dir, i, sg == 0 ? 1.0f : -1.0f);
                    float d = dot(dir, p);
                    if (d > best) { best = d; sup = p; }
                }
            }
            if (sg == 0) set_coord(s.localAabbMax, i, coord(sup, i) + m);
            else set_coord(s.localAabbMin, i, coord(sup, i) - m);
        }
    }
}

// OptimizedBvh.walkStacklessQuantizedTree (java:940-997) with testQuantizedAabbAgainstQuantizedAabb
// (java:563-585) over the query box quantized by quantizeWithClamp.
void mesh_overlapping_triangles(const MeshData& m, V3 aabbMin, V3 aabbMax, std::vector<int>& out) {
    out.clear();
    QuantizedBvh& t = const_cast<QuantizedBvh&>(m.bvh);
    BvhBuild b{t, {}, {}};
    uint16_t qa[3], qb[3];
    b.quantize(aabbMin, qa);
    b.quantize(aabbMax, qb);
    int cur = 0;
    while (cur < t.curNodeIndex) {
        const uint16_t* q = &t.q[6 * cur];
        bool ov = !(qa[0] > q[3] || qb[0] < q[0]) && !(qa[2] > q[5] || qb[2] < q[2]) && !(qa[1] > q[4] || qb[1] < q[1]);
        bool leaf = t.escOrTri[cur] >= 0;
        if (leaf && ov) out.push_back(t.escOrTri[cur] & ((1 << 21) - 1));
        if (ov || leaf) cur++;
        else cur += -t.escOrTri[cur];
    }
}

}  // namespace jb
