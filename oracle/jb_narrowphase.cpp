// ORACLE (test infrastructure only): narrowphase of the reference, restated.
// Citations relative to src/com/bulletphysics/.
#include <vector>
#include <algorithm>
#include "jb_world.h"

namespace jb {

// ----------------------------------------------------------------------------------------
// VoronoiSimplexSolver (collision/narrowphase/VoronoiSimplexSolver.java)
// ----------------------------------------------------------------------------------------
struct SubSimplexResult {
    V3 closest{0, 0, 0};
    bool uA = false, uB = false, uC = false, uD = false;
    float bc[4] = {0, 0, 0, 0};
    bool degenerate = false;
    void resetUsed() { uA = uB = uC = uD = false; }
    void reset() { degenerate = false; setBC(0, 0, 0, 0); resetUsed(); }
    bool isValid() const { return bc[0] >= 0.0f && bc[1] >= 0.0f && bc[2] >= 0.0f && bc[3] >= 0.0f; }
    void setBC(float a, float b, float c, float d) { bc[0] = a; bc[1] = b; bc[2] = c; bc[3] = d; }
};

struct VoronoiSimplex {
    int numVertices = 0;
    V3 W[5], P[5], Q[5];
    V3 cachedP1{0, 0, 0}, cachedP2{0, 0, 0}, cachedV{0, 0, 0}, lastW{0, 0, 0};
    bool cachedValidClosest = false, needsUpdate = true;
    SubSimplexResult cachedBC;

    void reset() {   // VoronoiSimplexSolver.java:567-573
        cachedValidClosest = false;
        numVertices = 0;
        needsUpdate = true;
        lastW = v3(1e30f, 1e30f, 1e30f);
        cachedBC.reset();
    }
    void removeVertex(int index) {
        numVertices--;
        W[index] = W[numVertices];
        P[index] = P[numVertices];
        Q[index] = Q[numVertices];
    }
    void reduceVertices(const SubSimplexResult& u) {
        if (numVertices >= 4 && !u.uD) removeVertex(3);
        if (numVertices >= 3 && !u.uC) removeVertex(2);
        if (numVertices >= 2 && !u.uB) removeVertex(1);
        if (numVertices >= 1 && !u.uA) removeVertex(0);
    }
    void addVertex(V3 w, V3 p, V3 q) {
        lastW = w;
        needsUpdate = true;
        W[numVertices] = w; P[numVertices] = p; Q[numVertices] = q;
        numVertices++;
    }
    bool inSimplex(V3 w) const {
        bool found = false;
        for (int i = 0; i < numVertices; i++) if (v3_equals(W[i], w)) found = true;
        if (v3_equals(w, lastW)) return true;
        return found;
    }

    // VoronoiSimplexSolver.closestPtPointTriangle (java:267-370)
    static bool closestPtPointTriangle(V3 p, V3 a, V3 b, V3 c, SubSimplexResult& r) {
        r.resetUsed();
        V3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
        float d1 = dot(ab, ap), d2 = dot(ac, ap);
        if (d1 <= 0.0f && d2 <= 0.0f) { r.closest = a; r.uA = true; r.setBC(1, 0, 0, 0); return true; }
        V3 bp = sub(p, b);
        float d3 = dot(ab, bp), d4 = dot(ac, bp);
        if (d3 >= 0.0f && d4 <= d3) { r.closest = b; r.uB = true; r.setBC(0, 1, 0, 0); return true; }
        float vc = d1 * d4 - d3 * d2;
        if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
            float v = d1 / (d1 - d3);
            r.closest = v3(v * ab.x + a.x, v * ab.y + a.y, v * ab.z + a.z);
            r.uA = r.uB = true; r.setBC(1.0f - v, v, 0, 0); return true;
        }
        V3 cp = sub(p, c);
        float d5 = dot(ab, cp), d6 = dot(ac, cp);
        if (d6 >= 0.0f && d5 <= d6) { r.closest = c; r.uC = true; r.setBC(0, 0, 1, 0); return true; }
        float vb = d5 * d2 - d1 * d6;
        if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
            float w = d2 / (d2 - d6);
            r.closest = v3(w * ac.x + a.x, w * ac.y + a.y, w * ac.z + a.z);
            r.uA = r.uC = true; r.setBC(1.0f - w, 0, w, 0); return true;
        }
        float va = d3 * d6 - d5 * d4;
        if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
            float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            V3 t = sub(c, b);
            r.closest = v3(w * t.x + b.x, w * t.y + b.y, w * t.z + b.z);
            r.uB = r.uC = true; r.setBC(0, 1.0f - w, w, 0); return true;
        }
        float denom = 1.0f / (va + vb + vc);
        float v = vb * denom, w = vc * denom;
        V3 t1 = scl(ab, v), t2 = scl(ac, w);
        r.closest = v3(a.x + t1.x + t2.x, a.y + t1.y + t2.y, a.z + t1.z + t2.z);
        r.uA = r.uB = r.uC = true;
        r.setBC(1.0f - v - w, v, w, 0);
        return true;
    }
    // VoronoiSimplexSolver.pointOutsideOfPlane (java:373-403)
    static int pointOutsideOfPlane(V3 p, V3 a, V3 b, V3 c, V3 d) {
        V3 normal = crs(sub(b, a), sub(c, a));
        float signp = dot(sub(p, a), normal);
        float signd = dot(sub(d, a), normal);
        if (signd * signd < ((1e-4f) * (1e-4f))) return -1;
        return (signp * signd < 0.0f) ? 1 : 0;
    }
    // VoronoiSimplexSolver.closestPtPointTetrahedron (java:405-535)
    bool closestPtPointTetrahedron(V3 p, V3 a, V3 b, V3 c, V3 d, SubSimplexResult& fin) {
        SubSimplexResult tmp;
        tmp.reset();
        fin.closest = p;
        fin.resetUsed();
        fin.uA = fin.uB = fin.uC = fin.uD = true;
        int oABC = pointOutsideOfPlane(p, a, b, c, d);
        int oACD = pointOutsideOfPlane(p, a, c, d, b);
        int oADB = pointOutsideOfPlane(p, a, d, b, c);
        int oBDC = pointOutsideOfPlane(p, b, d, c, a);
        if (oABC < 0 || oACD < 0 || oADB < 0 || oBDC < 0) { fin.degenerate = true; return false; }
        if (oABC == 0 && oACD == 0 && oADB == 0 && oBDC == 0) return false;
        float best = 3.40282347e+38f;
        if (oABC != 0) {
            closestPtPointTriangle(p, a, b, c, tmp);
            V3 q = tmp.closest;
            V3 t = sub(q, p);
            float sq = dot(t, t);
            if (sq < best) {
                best = sq; fin.closest = q; fin.resetUsed();
                fin.uA = tmp.uA; fin.uB = tmp.uB; fin.uC = tmp.uC;
                fin.setBC(tmp.bc[0], tmp.bc[1], tmp.bc[2], 0);
            }
        }
        if (oACD != 0) {
            closestPtPointTriangle(p, a, c, d, tmp);
            V3 q = tmp.closest;
            V3 t = sub(q, p);
            float sq = dot(t, t);
            if (sq < best) {
                best = sq; fin.closest = q; fin.resetUsed();
                fin.uA = tmp.uA; fin.uC = tmp.uB; fin.uD = tmp.uC;
                fin.setBC(tmp.bc[0], 0, tmp.bc[1], tmp.bc[2]);
            }
        }
        if (oADB != 0) {
            closestPtPointTriangle(p, a, d, b, tmp);
            V3 q = tmp.closest;
            V3 t = sub(q, p);
            float sq = dot(t, t);
            if (sq < best) {
                best = sq; fin.closest = q; fin.resetUsed();
                fin.uA = tmp.uA; fin.uB = tmp.uC; fin.uD = tmp.uB;
                fin.setBC(tmp.bc[0], tmp.bc[2], 0, tmp.bc[1]);
            }
        }
        if (oBDC != 0) {
            closestPtPointTriangle(p, b, d, c, tmp);
            V3 q = tmp.closest;
            V3 t = sub(q, p);
            float sq = dot(t, t);
            if (sq < best) {
                best = sq; fin.closest = q; fin.resetUsed();
                fin.uB = tmp.uA; fin.uC = tmp.uC; fin.uD = tmp.uB;
                fin.setBC(0, tmp.bc[0], tmp.bc[2], tmp.bc[1]);
            }
        }
        return true;
    }
    // VoronoiSimplexSolver.updateClosestVectorAndPoints (java:98-265)
    bool updateClosestVectorAndPoints() {
        if (needsUpdate) {
            cachedBC.reset();
            needsUpdate = false;
            switch (numVertices) {
            case 0:
                cachedValidClosest = false;
                break;
            case 1:
                cachedP1 = P[0];
                cachedP2 = Q[0];
                cachedV = sub(cachedP1, cachedP2);
                cachedBC.reset();
                cachedBC.setBC(1, 0, 0, 0);
                cachedValidClosest = cachedBC.isValid();
                break;
            case 2: {
                V3 from = W[0], to = W[1];
                V3 diff = sub(v3(0, 0, 0), from);
                V3 v = sub(to, from);
                float t = dot(v, diff);
                if (t > 0) {
                    float dotVV = dot(v, v);
                    if (t < dotVV) {
                        t /= dotVV;
                        diff = sub(diff, scl(v, t));
                        cachedBC.uA = true; cachedBC.uB = true;
                    } else {
                        t = 1;
                        diff = sub(diff, v);
                        cachedBC.uB = true;
                    }
                } else {
                    t = 0;
                    cachedBC.uA = true;
                }
                cachedBC.setBC(1.0f - t, t, 0, 0);
                cachedP1 = add(P[0], scl(sub(P[1], P[0]), t));
                cachedP2 = add(Q[0], scl(sub(Q[1], Q[0]), t));
                cachedV = sub(cachedP1, cachedP2);
                reduceVertices(cachedBC);
                cachedValidClosest = cachedBC.isValid();
                break;
            }
            case 3: {
                closestPtPointTriangle(v3(0, 0, 0), W[0], W[1], W[2], cachedBC);
                V3 t1 = scl(P[0], cachedBC.bc[0]), t2 = scl(P[1], cachedBC.bc[1]), t3 = scl(P[2], cachedBC.bc[2]);
                cachedP1 = v3(t1.x + t2.x + t3.x, t1.y + t2.y + t3.y, t1.z + t2.z + t3.z);
                t1 = scl(Q[0], cachedBC.bc[0]); t2 = scl(Q[1], cachedBC.bc[1]); t3 = scl(Q[2], cachedBC.bc[2]);
                cachedP2 = v3(t1.x + t2.x + t3.x, t1.y + t2.y + t3.y, t1.z + t2.z + t3.z);
                cachedV = sub(cachedP1, cachedP2);
                reduceVertices(cachedBC);
                cachedValidClosest = cachedBC.isValid();
                break;
            }
            case 4: {
                bool sep = closestPtPointTetrahedron(v3(0, 0, 0), W[0], W[1], W[2], W[3], cachedBC);
                if (sep) {
                    V3 t1 = scl(P[0], cachedBC.bc[0]), t2 = scl(P[1], cachedBC.bc[1]);
                    V3 t3 = scl(P[2], cachedBC.bc[2]), t4 = scl(P[3], cachedBC.bc[3]);
                    cachedP1 = v3(t1.x + t2.x + t3.x + t4.x, t1.y + t2.y + t3.y + t4.y, t1.z + t2.z + t3.z + t4.z);
                    t1 = scl(Q[0], cachedBC.bc[0]); t2 = scl(Q[1], cachedBC.bc[1]);
                    t3 = scl(Q[2], cachedBC.bc[2]); t4 = scl(Q[3], cachedBC.bc[3]);
                    cachedP2 = v3(t1.x + t2.x + t3.x + t4.x, t1.y + t2.y + t3.y + t4.y, t1.z + t2.z + t3.z + t4.z);
                    cachedV = sub(cachedP1, cachedP2);
                    reduceVertices(cachedBC);
                } else {
                    if (cachedBC.degenerate) {
                        cachedValidClosest = false;
                    } else {
                        cachedValidClosest = true;
                        cachedV = v3(0, 0, 0);
                    }
                    break;
                }
                cachedValidClosest = cachedBC.isValid();
                break;
            }
            default:
                cachedValidClosest = false;
            }
        }
        return cachedValidClosest;
    }
    bool closest(V3& v) { bool ok = updateClosestVectorAndPoints(); v = cachedV; return ok; }
    void compute_points(V3& p1, V3& p2) { updateClosestVectorAndPoints(); p1 = cachedP1; p2 = cachedP2; }
};

// ----------------------------------------------------------------------------------------
// GjkEpaSolver (collision/narrowphase/GjkEpaSolver.java), index-based pools.
// ----------------------------------------------------------------------------------------
namespace epa {
static const int GJK_maxiterations = 128;
static const float GJK_insimplex_eps = 0.0001f;
static const float GJK_sqinsimplex_eps = GJK_insimplex_eps * GJK_insimplex_eps;
static const int EPA_maxiterations = 256;
static const float EPA_inface_eps = 0.01f;
static const float EPA_accuracy = 0.001f;
static const float cstInf = SIMD_INFINITY;
static const float cst2Pi = SIMD_2_PI;

struct Mkv { V3 w, r; };

struct Gjk {
    const Shape* shapes[2];
    M3 rot[2];
    V3 pos[2];
    Mkv simplex[5];
    V3 ray;
    int order = 0, iterations = 0;
    float margin = 0;
    bool failed = false;
    std::vector<V3> seenRays;   // the 64-bucket hash of the reference, as a set (membership only)

    V3 LocalSupport(V3 d, int i) const {   // GjkEpaSolver.java:193-202
        V3 tmp = mulMTv(d, rot[i]);
        V3 out = support_with_margin(*shapes[i], tmp);
        out = mulMv(out, rot[i]);
        return add(out, pos[i]);
    }
    void Support(V3 d, Mkv& v) const {      // GjkEpaSolver.java:204-220
        v.r = d;
        V3 t1 = LocalSupport(d, 0);
        V3 t2 = LocalSupport(scl(d, -1.0f), 1);
        v.w = sub(t1, t2);
        v.w.x += margin * d.x;
        v.w.y += margin * d.y;
        v.w.z += margin * d.z;
    }
    bool FetchSupport() {                   // GjkEpaSolver.java:222-241
        for (size_t k = 0; k < seenRays.size(); k++)
            if (v3_equals(seenRays[k], ray)) { --order; return false; }
        seenRays.push_back(ray);
        Support(ray, simplex[++order]);
        return dot(ray, simplex[order].w) > 0;
    }
    bool SolveSimplex2(V3 ao, V3 ab) {      // java:243-261
        if (dot(ab, ao) >= 0) {
            V3 cabo = crs(ab, ao);
            if (len2(cabo) > GJK_sqinsimplex_eps) ray = crs(cabo, ab);
            else return true;
        } else {
            order = 0;
            simplex[0] = simplex[1];
            ray = ao;
        }
        return false;
    }
    bool SolveSimplex3(V3 ao, V3 ab, V3 ac) { return SolveSimplex3a(ao, ab, ac, crs(ab, ac)); }
    bool SolveSimplex3a(V3 ao, V3 ab, V3 ac, V3 cabc) {   // java:272-307
        V3 t = crs(cabc, ab);
        V3 t2 = crs(cabc, ac);
        if (dot(t, ao) < -GJK_insimplex_eps) {
            order = 1;
            simplex[0] = simplex[1];
            simplex[1] = simplex[2];
            return SolveSimplex2(ao, ab);
        } else if (dot(t2, ao) > +GJK_insimplex_eps) {
            order = 1;
            simplex[1] = simplex[2];
            return SolveSimplex2(ao, ac);
        } else {
            float d = dot(cabc, ao);
            if (std::fabs(d) > GJK_insimplex_eps) {
                if (d > 0) ray = cabc;
                else {
                    ray = scl(cabc, -1.0f);
                    Mkv s = simplex[0];
                    simplex[0] = simplex[1];
                    simplex[1] = s;
                }
                return false;
            }
            return true;
        }
    }
    bool SolveSimplex4(V3 ao, V3 ab, V3 ac, V3 ad) {      // java:309-345
        V3 t = crs(ab, ac), t2 = crs(ac, ad), t3 = crs(ad, ab);
        if (dot(t, ao) > GJK_insimplex_eps) {
            order = 2;
            simplex[0] = simplex[1]; simplex[1] = simplex[2]; simplex[2] = simplex[3];
            return SolveSimplex3a(ao, ab, ac, t);
        } else if (dot(t2, ao) > GJK_insimplex_eps) {
            order = 2;
            simplex[2] = simplex[3];
            return SolveSimplex3a(ao, ac, ad, t2);
        } else if (dot(t3, ao) > GJK_insimplex_eps) {
            order = 2;
            simplex[1] = simplex[0]; simplex[0] = simplex[2]; simplex[2] = simplex[3];
            return SolveSimplex3a(ao, ad, ab, t3);
        }
        return true;
    }
    bool SearchOrigin() {                   // java:354-420, initial ray (1,0,0)
        iterations = 0;
        order = -1;
        failed = false;
        ray = nor(v3(1, 0, 0));
        seenRays.clear();
        FetchSupport();
        ray = scl(simplex[0].w, -1.0f);
        for (; iterations < GJK_maxiterations; ++iterations) {
            float rl = len(ray);
            ray = scl(ray, 1.0f / (rl > 0.0f ? rl : 1.0f));
            if (FetchSupport()) {
                bool found = false;
                switch (order) {
                case 1:
                    found = SolveSimplex2(scl(simplex[1].w, -1.0f), sub(simplex[0].w, simplex[1].w));
                    break;
                case 2:
                    found = SolveSimplex3(scl(simplex[2].w, -1.0f), sub(simplex[1].w, simplex[2].w), sub(simplex[0].w, simplex[2].w));
                    break;
                case 3:
                    found = SolveSimplex4(scl(simplex[3].w, -1.0f), sub(simplex[2].w, simplex[3].w),
                                          sub(simplex[1].w, simplex[3].w), sub(simplex[0].w, simplex[3].w));
                    break;
                }
                if (found) return true;
            } else {
                return false;
            }
        }
        failed = true;
        return false;
    }
    bool EncloseOrigin() {                  // java:422-505
        switch (order) {
        case 0:
            break;
        case 1: {
            V3 ab = sub(simplex[1].w, simplex[0].w);
            // The port evaluates b[i].set(ab).crs(b[i]): the axis is overwritten by ab before the
            // cross product, so all three candidates are ab x ab (GjkEpaSolver.java:433-438).
            V3 b[3];
            for (int i = 0; i < 3; i++) b[i] = crs(ab, ab);
            float m[3] = {len2(b[0]), len2(b[1]), len2(b[2])};
            Quat q = q_axis_angle(nor(ab), cst2Pi / 3.0f);
            M3 r = m3_from_quat(q);
            V3 w = b[m[0] > m[1] ? (m[0] > m[2] ? 0 : 2) : (m[1] > m[2] ? 1 : 2)];
            Support(nor(w), simplex[4]);
            w = mulMv(w, r);
            Support(nor(w), simplex[2]);
            w = mulMv(w, r);
            Support(nor(w), simplex[3]);
            w = mulMv(w, r);
            order = 4;
            return true;
        }
        case 2: {
            V3 n = nor(crs(sub(simplex[1].w, simplex[0].w), sub(simplex[2].w, simplex[0].w)));
            Support(n, simplex[3]);
            Support(scl(n, -1.0f), simplex[4]);
            order = 4;
            return true;
        }
        case 3:
        case 4:
            return true;
        }
        return false;
    }
};

static const int mod3[5] = {0, 1, 2, 0, 1};
static const int tet_fidx[4][3] = {{2, 1, 0}, {3, 0, 1}, {3, 1, 2}, {3, 2, 0}};
static const int tet_eidx[6][4] = {{0, 0, 2, 1}, {0, 1, 1, 1}, {0, 2, 3, 1}, {1, 0, 3, 2}, {2, 0, 1, 2}, {3, 0, 2, 2}};
static const int hex_fidx[6][3] = {{2, 0, 4}, {4, 1, 2}, {1, 4, 0}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
static const int hex_eidx[9][4] = {{0, 0, 4, 0}, {0, 1, 2, 1}, {0, 2, 1, 2}, {1, 1, 5, 2}, {1, 0, 2, 0},
                                   {2, 2, 3, 2}, {3, 1, 5, 0}, {3, 0, 4, 2}, {5, 1, 4, 1}};

struct Face { int v[3]; int f[3]; int e[3]; V3 n; float d; int mark; int prev, next; };

struct Epa {                                  // GjkEpaSolver.EPA (java:538-858)
    Gjk* gjk;
    std::vector<Mkv> mkv;
    std::vector<Face> faces;
    int root = -1, nfaces = 0, iterations = 0;
    V3 nearest[2];
    V3 normal{0, 0, 0};
    float depth = 0;
    bool failed = false;

    V3 GetCoordinates(const Face& f) const {
        V3 o = scl(f.n, -f.d);
        float a0 = len(crs(sub(mkv[f.v[0]].w, o), sub(mkv[f.v[1]].w, o)));
        float a1 = len(crs(sub(mkv[f.v[1]].w, o), sub(mkv[f.v[2]].w, o)));
        float a2 = len(crs(sub(mkv[f.v[2]].w, o), sub(mkv[f.v[0]].w, o)));
        float sm = a0 + a1 + a2;
        return scl(v3(a1, a2, a0), 1.0f / (sm > 0.0f ? sm : 1.0f));
    }
    int FindBest() const {
        int bf = -1;
        if (root >= 0) {
            int cf = root;
            float bd = cstInf;
            do {
                if (faces[cf].d < bd) { bd = faces[cf].d; bf = cf; }
            } while ((cf = faces[cf].next) >= 0);
        }
        return bf;
    }
    bool Set(Face& f, int a, int b, int c) const {
        V3 aw = mkv[a].w, bw = mkv[b].w, cw = mkv[c].w;
        V3 nrm = crs(sub(bw, aw), sub(cw, aw));
        float l = len(nrm);
        V3 t1 = crs(aw, bw), t2 = crs(bw, cw), t3 = crs(cw, aw);
        bool valid = (dot(t1, nrm) >= -EPA_inface_eps) && (dot(t2, nrm) >= -EPA_inface_eps) && (dot(t3, nrm) >= -EPA_inface_eps);
        f.v[0] = a; f.v[1] = b; f.v[2] = c;
        f.mark = 0;
        f.n = scl(nrm, 1.0f / (l > 0.0f ? l : cstInf));
        f.d = jmax(0.0f, -dot(f.n, aw));
        return valid;
    }
    int NewFace(int a, int b, int c) {
        Face nf;
        for (int i = 0; i < 3; i++) { nf.f[i] = -1; nf.e[i] = 0; }
        int id = (int)faces.size();
        bool ok = Set(nf, a, b, c);
        faces.push_back(nf);
        if (ok) {
            if (root >= 0) faces[root].prev = id;
            faces[id].prev = -1;
            faces[id].next = root;
            root = id;
            ++nfaces;
        } else {
            faces[id].prev = faces[id].next = -1;
        }
        return id;
    }
    void Detach(int fi) {
        Face& f = faces[fi];
        if (f.prev >= 0 || f.next >= 0) {
            --nfaces;
            if (fi == root) {
                root = f.next;
                if (root >= 0) faces[root].prev = -1;   // the reference dereferences null here (unreachable in practice)
            } else {
                if (f.next < 0) faces[f.prev].next = -1;
                else { faces[f.prev].next = f.next; faces[f.next].prev = f.prev; }
            }
            f.prev = f.next = -1;
        }
    }
    void Link(int f0, int e0, int f1, int e1) {
        faces[f0].f[e0] = f1; faces[f1].e[e1] = e0;
        faces[f1].f[e1] = f0; faces[f0].e[e0] = e1;
    }
    int SupportNew(V3 w) {
        Mkv v;
        gjk->Support(w, v);
        mkv.push_back(v);
        return (int)mkv.size() - 1;
    }
    int BuildHorizon(int markid, int w, int f, int e, int& cf, int& ff) {   // java:658-683
        int ne = 0;
        if (faces[f].mark != markid) {
            int e1 = mod3[e + 1];
            if ((dot(faces[f].n, mkv[w].w) + faces[f].d) > 0) {
                int nf = NewFace(faces[f].v[e1], faces[f].v[e], w);
                Link(nf, 0, f, e);
                if (cf >= 0) Link(cf, 1, nf, 2);
                else ff = nf;
                cf = nf;
                ne = 1;
            } else {
                int e2 = mod3[e + 2];
                Detach(f);
                faces[f].mark = markid;
                ne += BuildHorizon(markid, w, faces[f].f[e1], faces[f].e[e1], cf, ff);
                ne += BuildHorizon(markid, w, faces[f].f[e2], faces[f].e[e2], cf, ff);
            }
        }
        return ne;
    }
    float EvaluatePD(float accuracy) {        // java:689-851
        int bestface = -1;
        int markid = 1;
        depth = -cstInf;
        normal = v3(0, 0, 0);
        root = -1;
        nfaces = 0;
        iterations = 0;
        failed = false;
        if (gjk->EncloseOrigin()) {
            const int(*pf)[3] = nullptr;
            const int(*pe)[4] = nullptr;
            int nfidx = 0, neidx = 0;
            if (gjk->order == 3) { pf = tet_fidx; nfidx = 4; pe = tet_eidx; neidx = 6; }
            else if (gjk->order == 4) { pf = hex_fidx; nfidx = 6; pe = hex_eidx; neidx = 9; }
            int base = (int)mkv.size();
            for (int i = 0; i <= gjk->order; ++i) mkv.push_back(gjk->simplex[i]);
            int basefaces[6];
            for (int i = 0; i < nfidx; ++i) basefaces[i] = NewFace(base + pf[i][0], base + pf[i][1], base + pf[i][2]);
            for (int i = 0; i < neidx; ++i) Link(basefaces[pe[i][0]], pe[i][1], basefaces[pe[i][2]], pe[i][3]);
        }
        if (0 == nfaces) return depth;
        for (; iterations < EPA_maxiterations; ++iterations) {
            int bf = FindBest();
            if (bf >= 0) {
                int w = SupportNew(scl(faces[bf].n, -1.0f));
                float d = dot(faces[bf].n, mkv[w].w) + faces[bf].d;
                bestface = bf;
                if (d < -accuracy) {
                    int cf = -1, ff = -1;
                    int nf = 0;
                    Detach(bf);
                    faces[bf].mark = ++markid;
                    for (int i = 0; i < 3; ++i) nf += BuildHorizon(markid, w, faces[bf].f[i], faces[bf].e[i], cf, ff);
                    if (nf <= 2) break;
                    Link(cf, 1, ff, 2);
                } else {
                    break;
                }
            } else {
                break;
            }
        }
        if (bestface >= 0) {
            const Face& bfc = faces[bestface];
            V3 b = GetCoordinates(bfc);
            normal = bfc.n;
            depth = jmax(0.0f, bfc.d);
            V3 feat[2][3];
            for (int i = 0; i < 2; ++i) {
                float s = i != 0 ? -1.0f : 1.0f;
                for (int j = 0; j < 3; ++j) feat[i][j] = gjk->LocalSupport(scl(mkv[bfc.v[j]].r, s), i);
            }
            for (int i = 0; i < 2; i++) {
                V3 t1 = scl(feat[i][0], b.x), t2 = scl(feat[i][1], b.y), t3 = scl(feat[i][2], b.z);
                nearest[i] = v3(t1.x + t2.x + t3.x, t1.y + t2.y + t3.y, t1.z + t2.z + t3.z);
            }
        } else {
            failed = true;
        }
        return depth;
    }
};

// GjkEpaSolver.collide + GjkEpaPenetrationDepthSolver.calcPenDepth
// (GjkEpaSolver.java:864-907, GjkEpaPenetrationDepthSolver.java:41-63)
static bool calc_pen_depth(const Shape& s0, const Xf& t0, const Shape& s1, const Xf& t1, V3& wA, V3& wB) {
    Gjk gjk;
    gjk.shapes[0] = &s0; gjk.rot[0] = t0.b; gjk.pos[0] = t0.o;
    gjk.shapes[1] = &s1; gjk.rot[1] = t1.b; gjk.pos[1] = t1.o;
    gjk.margin = 0.0f + EPA_accuracy;
    gjk.failed = false;
    bool collide = gjk.SearchOrigin();
    if (collide) {
        Epa e;
        e.gjk = &gjk;
        float pd = e.EvaluatePD(EPA_accuracy);
        if (pd > 0) {
            wA = e.nearest[0];
            wB = e.nearest[1];
            return true;
        }
    }
    return false;
}
}  // namespace epa

// ----------------------------------------------------------------------------------------
// GjkPairDetector.getClosestPoints (collision/narrowphase/GjkPairDetector.java:73-316)
// ----------------------------------------------------------------------------------------
GjkOut gjk_closest_points(const Shape& sa, const Xf& tA, const Shape& sb, const Xf& tB, float maxDist2, bool withEpa) {
    static const float REL_ERROR2 = 1.0e-6f;
    GjkOut out;
    out.valid = false;
    out.usedEpa = 0;
    float distance = 0.0f;
    V3 normalInB = v3(0, 0, 0), pointOnA{0, 0, 0}, pointOnB{0, 0, 0};
    Xf lA = tA, lB = tB;
    V3 positionOffset = scl(add(lA.o, lB.o), 0.5f);
    lA.o = sub(lA.o, positionOffset);
    lB.o = sub(lB.o, positionOffset);
    float marginA = sa.getMargin(), marginB = sb.getMargin();
    int curIter = 0;
    const int gGjkMaxIter = 1000;
    V3 sep = v3(0, 1, 0);
    bool isValid = false, checkSimplex = false, checkPenetration = true;
    int degenerate = 0;
    float squaredDistance = SIMD_INFINITY;
    float delta = 0.0f;
    float margin = marginA + marginB;
    VoronoiSimplex simplex;
    simplex.reset();
    for (;;) {
        V3 sepA = mulMTv(scl(sep, -1.0f), tA.b);
        V3 sepB = mulMTv(sep, tB.b);
        V3 pInA = support_without_margin(sa, sepA);
        V3 qInB = support_without_margin(sb, sepB);
        V3 pW = xf_apply(lA, pInA);
        V3 qW = xf_apply(lB, qInB);
        V3 w = sub(pW, qW);
        delta = dot(sep, w);
        if ((delta > 0.0f) && (delta * delta > squaredDistance * maxDist2)) { checkPenetration = false; break; }
        if (simplex.inSimplex(w)) { degenerate = 1; checkSimplex = true; break; }
        float f0 = squaredDistance - delta;
        float f1 = squaredDistance * REL_ERROR2;
        if (f0 <= f1) { if (f0 <= 0.0f) degenerate = 2; checkSimplex = true; break; }
        simplex.addVertex(w, pW, qW);
        if (!simplex.closest(sep)) { degenerate = 3; checkSimplex = true; break; }
        if (len2(sep) < REL_ERROR2) { degenerate = 6; checkSimplex = true; break; }
        float previous = squaredDistance;
        squaredDistance = len2(sep);
        if (previous - squaredDistance <= FLT_EPS * previous) {
            sep = simplex.cachedV;
            checkSimplex = true;
            break;
        }
        if (curIter++ > gGjkMaxIter) break;
        if (simplex.numVertices == 4) { sep = simplex.cachedV; break; }
    }
    if (checkSimplex) {
        simplex.compute_points(pointOnA, pointOnB);
        normalInB = sub(pointOnA, pointOnB);
        float lenSqr = len2(sep);
        if (lenSqr < 0.0001f) degenerate = 5;
        if (lenSqr > FLT_EPS * FLT_EPS) {
            float rlen = 1.0f / jsqrt(lenSqr);
            normalInB = scl(normalInB, rlen);
            float s = jsqrt(squaredDistance);
            pointOnA = sub(pointOnA, scl(sep, marginA / s));
            pointOnB = add(pointOnB, scl(sep, marginB / s));
            distance = (1.0f / rlen) - margin;
            isValid = true;
        }
    }
    bool catchDegeneratePenetrationCase = (degenerate != 0 && ((distance + margin) < 0.01f));
    if (withEpa && checkPenetration && (!isValid || catchDegeneratePenetrationCase)) {
        out.usedEpa = 1;
        V3 tA2, tB2;
        if (epa::calc_pen_depth(sa, lA, sb, lB, tA2, tB2)) {
            V3 tn = sub(tB2, tA2);
            float lenSqr = len2(tn);
            if (lenSqr > (FLT_EPS * FLT_EPS)) {
                tn = scl(tn, 1.0f / jsqrt(lenSqr));
                float distance2 = -len(sub(tA2, tB2));
                if (!isValid || (distance2 < distance)) {
                    distance = distance2;
                    pointOnA = tA2;
                    pointOnB = tB2;
                    normalInB = tn;
                    isValid = true;
                }
            }
        }
    }
    out.valid = isValid;
    if (isValid) {
        out.normal = normalInB;
        out.pointOnB = add(pointOnB, positionOffset);
        out.distance = distance;
    }
    return out;
}

// ----------------------------------------------------------------------------------------
// PersistentManifold + ManifoldResult
// ----------------------------------------------------------------------------------------
// PersistentManifold.sortCachedPoints (PersistentManifold.java:83-156)
static int sort_cached_points(const Manifold& m, const ManifoldPoint& pt) {
    int maxPenetrationIndex = -1;
    float maxPenetration = pt.distance;
    for (int i = 0; i < 4; i++)
        if (m.pts[i].distance < maxPenetration) { maxPenetrationIndex = i; maxPenetration = m.pts[i].distance; }
    float res0 = 0, res1 = 0, res2 = 0, res3 = 0;
    if (maxPenetrationIndex != 0) res0 = len2(crs(sub(pt.localA, m.pts[1].localA), sub(m.pts[3].localA, m.pts[2].localA)));
    if (maxPenetrationIndex != 1) res1 = len2(crs(sub(pt.localA, m.pts[0].localA), sub(m.pts[3].localA, m.pts[2].localA)));
    if (maxPenetrationIndex != 2) res2 = len2(crs(sub(pt.localA, m.pts[0].localA), sub(m.pts[3].localA, m.pts[1].localA)));
    if (maxPenetrationIndex != 3) res3 = len2(crs(sub(pt.localA, m.pts[0].localA), sub(m.pts[2].localA, m.pts[1].localA)));
    // VectorUtil.closestAxis4 -> maxAxis4 of the absolute values
    float v[4] = {std::fabs(res0), std::fabs(res1), std::fabs(res2), std::fabs(res3)};
    int maxIndex = -1;
    float maxVal = -1e30f;
    for (int i = 0; i < 4; i++) if (v[i] > maxVal) { maxIndex = i; maxVal = v[i]; }
    return maxIndex;
}

// PersistentManifold.removeContactPoint (PersistentManifold.java:259-278)
static void remove_contact_point(Manifold& m, int index) {
    int last = m.n - 1;
    if (index != last) {
        m.pts[index] = m.pts[last];
        m.pts[last].appliedImpulse = 0;
        m.pts[last].latInit = false;
        m.pts[last].lat1 = 0;
        m.pts[last].lat2 = 0;
        m.pts[last].lifeTime = 0;
    }
    m.n--;
}

// PersistentManifold.refreshContactPoints (PersistentManifold.java:312-372)
static void refresh_contact_points(Manifold& m, const Xf& trA, const Xf& trB, float cbt) {
    for (int i = m.n - 1; i >= 0; i--) {
        ManifoldPoint& p = m.pts[i];
        p.worldA = xf_apply(trA, p.localA);
        p.worldB = xf_apply(trB, p.localB);
        p.distance = dot(sub(p.worldA, p.worldB), p.normal);
        p.lifeTime++;
    }
    for (int i = m.n - 1; i >= 0; i--) {
        ManifoldPoint& p = m.pts[i];
        if (!(p.distance <= cbt)) {
            remove_contact_point(m, i);
        } else {
            V3 projectedPoint = sub(p.worldA, scl(p.normal, p.distance));
            V3 projectedDifference = sub(p.worldB, projectedPoint);
            float distance2d = dot(projectedDifference, projectedDifference);
            if (distance2d > cbt * cbt) remove_contact_point(m, i);
        }
    }
}

// ManifoldResult.addContactPoint (collision/dispatch/ManifoldResult.java:92-157)
static void manifold_add_contact(World& w, Manifold& m, int col0, int col1, V3 normalOnB, V3 pointInWorld, float depth) {
    const float cbt = w.cfg.contactBreakingThreshold;
    if (depth > cbt) return;
    const Body& b0 = w.bodies[col0];
    const Body& b1 = w.bodies[col1];
    bool isSwapped = m.body0 != col0;
    V3 pointA = add(scl(normalOnB, depth), pointInWorld);
    V3 localA, localB;
    if (isSwapped) {
        localA = xf_invXform(b1.xf, pointA);
        localB = xf_invXform(b0.xf, pointInWorld);
    } else {
        localA = xf_invXform(b0.xf, pointA);
        localB = xf_invXform(b1.xf, pointInWorld);
    }
    ManifoldPoint np;   // ManifoldPoint.init (ManifoldPoint.java:73-86); lateral dirs are never read before re-initialisation
    np.localA = localA; np.localB = localB; np.normal = normalOnB; np.distance = depth;
    np.worldA = pointA; np.worldB = pointInWorld;
    // PersistentManifold.getCacheEntry (PersistentManifold.java:214-233)
    float shortest = cbt * cbt;
    int nearest = -1;
    for (int i = 0; i < m.n; i++) {
        V3 d = sub(m.pts[i].localA, np.localA);
        float dd = dot(d, d);
        if (dd < shortest) { shortest = dd; nearest = i; }
    }
    // ManifoldResult.calculateCombinedFriction / Restitution (ManifoldResult.java:160-175)
    float fr = b0.friction * b1.friction;
    if (fr < -10.0f) fr = -10.0f;
    if (fr > 10.0f) fr = 10.0f;
    np.friction = fr;
    np.restitution = b0.restitution * b1.restitution;
    if (nearest >= 0) {
        // PersistentManifold.replaceContactPoint keeps impulses and lifetime (PersistentManifold.java:280-305)
        ManifoldPoint& o = m.pts[nearest];
        int life = o.lifeTime;
        float ai = o.appliedImpulse, l1 = o.lat1, l2 = o.lat2;
        V3 d1 = o.latDir1, d2 = o.latDir2;
        o = np;
        o.appliedImpulse = ai; o.lat1 = l1; o.lat2 = l2; o.lifeTime = life;
        o.latDir1 = d1; o.latDir2 = d2;   // stale values, unused while latInit == false
    } else {
        // PersistentManifold.addManifoldPoint (PersistentManifold.java:235-257)
        int ins = m.n;
        if (ins == 4) ins = sort_cached_points(m, np);
        else m.n++;
        m.pts[ins] = np;
    }
}

static void manifold_refresh(World& w, Manifold& m) {   // ManifoldResult.refreshContactPoints (java:177-191)
    if (m.n == 0) return;
    refresh_contact_points(m, w.bodies[m.body0].xf, w.bodies[m.body1].xf, w.cfg.contactBreakingThreshold);
}

// ----------------------------------------------------------------------------------------
// Collision algorithms
// ----------------------------------------------------------------------------------------
// A collision object as a collision algorithm sees it: the shape and world transform it holds
// while the algorithm runs (CompoundCollisionAlgorithm swaps in a child with orgTrans *
// childTrans, ConvexTriangleCallback a TriangleShape), and its body.
struct CObj {
    const Shape* s;
    Xf xf;
    int body;
};

// SphereSphereCollisionAlgorithm.processCollision (java:73-134)
static void sphere_sphere(World& w, Manifold& m, int col0, int col1, const CObj& A, const CObj& B) {
    V3 diff = sub(A.xf.o, B.xf.o);
    float l = len(diff);
    float r0 = A.s->getMargin();
    float r1 = B.s->getMargin();
    if (l > (r0 + r1)) { manifold_refresh(w, m); return; }
    float dist = l - (r0 + r1);
    V3 n = v3(1, 0, 0);
    if (l > FLT_EPS) n = scl(diff, 1.0f / l);
    V3 pos1 = add(B.xf.o, scl(n, r1));
    manifold_add_contact(w, m, col0, col1, n, pos1, dist);
    manifold_refresh(w, m);
}

// ConvexPlaneCollisionAlgorithm.processCollision (java:75-136)
static void convex_plane(World& w, Manifold& m, int col0, int col1, const CObj& C, const CObj& P) {
    const Shape& cs = *C.s;
    const Shape& ps = *P.s;
    V3 pn = ps.planeNormal;
    float pc = ps.planeConstant;
    Xf planeInConvex = xf_mul(xf_inverse(C.xf), P.xf);
    Xf convexInPlane = xf_mul(xf_inverse(P.xf), C.xf);
    V3 dir = mulMv(scl(pn, -1.0f), planeInConvex.b);
    V3 vtx = support_with_margin(cs, dir);
    V3 vtxInPlane = xf_apply(convexInPlane, vtx);
    float distance = dot(pn, vtxInPlane) - pc;
    V3 proj = sub(vtxInPlane, scl(pn, distance));
    V3 vtxWorld = xf_apply(P.xf, proj);
    bool hasCollision = distance < w.cfg.contactBreakingThreshold;
    if (hasCollision) {
        V3 normalOnB = mulMv(pn, P.xf.b);
        manifold_add_contact(w, m, col0, col1, normalOnB, vtxWorld, distance);
    }
    if (m.n != 0) manifold_refresh(w, m);
}

// GjkPairDetector between A and B as ConvexConvexAlgorithm.processCollision (java:90-139) runs it;
// adds the point, without the refresh.
static void convex_convex_point(World& w, Manifold& m, int col0, int col1, const CObj& A, const CObj& B) {
    float md = A.s->getMargin() + B.s->getMargin() + w.cfg.contactBreakingThreshold;
    md *= md;
    w.counters.gjk++;
    GjkOut g = gjk_closest_points(*A.s, A.xf, *B.s, B.xf, md);
    if (g.usedEpa) w.counters.epa++;
    if (g.valid) manifold_add_contact(w, m, col0, col1, g.normal, g.pointOnB, g.distance);
}

// ConvexConvexAlgorithm.processCollision (java:90-139) with its own manifold
static void convex_convex(World& w, Manifold& m, int col0, int col1, const CObj& A, const CObj& B) {
    convex_convex_point(w, m, col0, col1, A, B);
    manifold_refresh(w, m);
}

// ConvexConcaveCollisionAlgorithm.processCollision (java:65-97): ConvexTriangleCallback's query box
// (the convex shape's aabb in the mesh's space widened by the mesh margin,
// ConvexTriangleCallback.setTimeStepAndCounters java:82-104), the mesh's triangles overlapping it
// in walk order, each collided as a TriangleShape with the mesh margin by ConvexConvexAlgorithm
// into the shared manifold (ConvexTriangleCallback.processTriangle java:109-166), then one refresh.
static void convex_concave(World& w, Manifold& m, int col0, int col1, const CObj& C, const CObj& T) {
    Xf convexInTri = xf_mul(xf_inverse(T.xf), C.xf);
    V3 mn, mx;
    shape_aabb(*C.s, convexInTri, mn, mx);
    float mt = T.s->getMargin();
    mx = add(mx, v3(mt, mt, mt));
    mn = sub(mn, v3(mt, mt, mt));
    std::vector<int> tris;
    mesh_overlapping_triangles(*T.s->mesh, mn, mx, tris);
    Shape tm;
    tm.type = TRIANGLE;
    tm.collisionMargin = mt;
    for (int t : tris) {
        for (int k = 0; k < 3; k++) tm.tri[k] = T.s->mesh->tri[3 * t + k];
        convex_convex_point(w, m, col0, col1, C, CObj{&tm, T.xf, T.body});
    }
    manifold_refresh(w, m);
}

// CollisionDispatcher.needsCollision (java:198-223)
static bool needs_collision(const Body& a, const Body& b) {
    if (!a.isActive() && !b.isActive()) return false;
    return true;
}

// CompoundShapeChild i of a compound object: orgTrans * childTrans (CompoundCollisionAlgorithm.
// processCollision java:101-124)
static CObj compound_child(const CObj& c, int i) {
    return CObj{&c.s->children[i], xf_mul(c.xf, c.s->childXf[i]), c.body};
}

// The two leaf objects a pair's algorithm collides, in the algorithm's order.  col0/col1 are the
// lower/higher uid (proxy0/proxy1 of the BroadphasePair).  A pair with a compound body is one
// key per child combination: the combination's algorithm is the one CompoundCollisionAlgorithm.
// init finds for the compound's child against the other object - the compound side first, and
// with two compounds the higher body's child first (the swapped algorithm that the lower body's
// child finds against the higher compound).
static void pair_objects(const World& w, uint64_t key, CObj& f, CObj& g) {
    int a = key_owner(key), b = key_partner(key), sub = key_sub(key);
    int col0 = a < b ? a : b, col1 = a < b ? b : a;
    const Body& B0 = w.bodies[col0];
    const Body& B1 = w.bodies[col1];
    const Shape& S0 = w.shapes[B0.shape];
    const Shape& S1 = w.shapes[B1.shape];
    CObj o0{&S0, B0.xf, col0}, o1{&S1, B1.xf, col1};
    f = o0;
    g = o1;
    if (S0.isCompound() || S1.isCompound()) {
        int n1 = S1.isCompound() ? (int)S1.children.size() : 1;
        CObj l0 = S0.isCompound() ? compound_child(o0, sub / n1) : o0;
        CObj l1 = S1.isCompound() ? compound_child(o1, sub % n1) : o1;
        if (S1.isCompound()) { f = l1; g = l0; }
        else { f = l0; g = l1; }
    }
}

// DefaultCollisionConfiguration.getCollisionAlgorithmCreateFunc (java:160-215) over the leaf shape
// types: the algorithm kind, and the bodies of the manifold it creates (convex before plane or
// mesh, else the algorithm's order).  Kind 0: EmptyAlgorithm (two concave shapes), no manifold.
enum { ALG_EMPTY = 0, ALG_SPHERE_SPHERE, ALG_CONVEX_PLANE, ALG_PLANE_CONVEX, ALG_CONVEX_CONVEX, ALG_CONVEX_CONCAVE,
       ALG_CONCAVE_CONVEX };
static int algorithm_kind(const CObj& f, const CObj& g, int& mb0, int& mb1) {
    const Shape& F = *f.s;
    const Shape& G = *g.s;
    int k = ALG_EMPTY;
    if (F.type == SPHERE && G.type == SPHERE) k = ALG_SPHERE_SPHERE;
    else if (F.isConvex() && G.type == STATIC_PLANE) k = ALG_CONVEX_PLANE;
    else if (G.isConvex() && F.type == STATIC_PLANE) k = ALG_PLANE_CONVEX;
    else if (F.isConvex() && G.isConvex()) k = ALG_CONVEX_CONVEX;
    else if (F.isConvex() && G.isConcave()) k = ALG_CONVEX_CONCAVE;
    else if (G.isConvex() && F.isConcave()) k = ALG_CONCAVE_CONVEX;
    bool swapped = k == ALG_PLANE_CONVEX || k == ALG_CONCAVE_CONVEX;
    mb0 = swapped ? g.body : f.body;
    mb1 = swapped ? f.body : g.body;
    return k;
}

bool pair_manifold_bodies(const World& w, uint64_t key, int& mb0, int& mb1) {
    CObj f, g;
    pair_objects(w, key, f, g);
    return algorithm_kind(f, g, mb0, mb1) != ALG_EMPTY;
}

// DefaultNearCallback.handleCollision (collision/dispatch/DefaultNearCallback.java:39-66) for one
// pair: needsCollision, the algorithm (and its manifold) on first contact, processCollision.
void process_pair(World& w, int pi) {
    uint64_t key = w.pairKeys[pi];
    int a = key_owner(key), b = key_partner(key);
    int col0 = a < b ? a : b, col1 = a < b ? b : a;
    if (!needs_collision(w.bodies[col0], w.bodies[col1])) return;
    CObj f, g;
    pair_objects(w, key, f, g);
    int mb0, mb1;
    int kind = algorithm_kind(f, g, mb0, mb1);
    if (kind == ALG_EMPTY) return;
    Manifold& m = w.pairMf[pi];
    if (!w.pairHasAlgo[pi]) { w.pairHasAlgo[pi] = 1; m = Manifold(); m.body0 = mb0; m.body1 = mb1; }
    switch (kind) {
    case ALG_SPHERE_SPHERE: sphere_sphere(w, m, col0, col1, f, g); break;
    case ALG_CONVEX_PLANE: convex_plane(w, m, col0, col1, f, g); break;
    case ALG_PLANE_CONVEX: convex_plane(w, m, col0, col1, g, f); break;
    case ALG_CONVEX_CONVEX: convex_convex(w, m, col0, col1, f, g); break;
    case ALG_CONVEX_CONCAVE: convex_concave(w, m, col0, col1, f, g); break;
    case ALG_CONCAVE_CONVEX: convex_concave(w, m, col0, col1, g, f); break;
    }
}


// ----------------------------------------------------------------------------------------
// CollisionWorld.rayTest with a ClosestRayResultCallback (collision/dispatch/CollisionWorld.java:
// 553-591 and rayTestSingle 260-331, ClosestRayResultCallback 697-729)
// ----------------------------------------------------------------------------------------
// AabbUtil2.outcode (linearmath/AabbUtil2.java:40-43)
static int outcode(V3 p, V3 h) {
    return (p.x < -h.x ? 0x01 : 0x0) | (p.x > h.x ? 0x08 : 0x0) | (p.y < -h.y ? 0x02 : 0x0) | (p.y > h.y ? 0x10 : 0x0) |
           (p.z < -h.z ? 0x4 : 0x0) | (p.z > h.z ? 0x20 : 0x0);
}

// AabbUtil2.rayAabb (linearmath/AabbUtil2.java:45-104): param in = the largest fraction
// accepted, out = the entry fraction.
static bool ray_aabb(V3 from, V3 to, V3 mn, V3 mx, float& param) {
    V3 he = scl(sub(mx, mn), 0.5f);
    V3 c = scl(add(mx, mn), 0.5f);
    V3 source = sub(from, c), target = sub(to, c);
    int so = outcode(source, he), to_ = outcode(target, he);
    if ((so & to_) != 0) return false;
    float enter = 0.0f, exit = param;
    V3 r = sub(target, source);
    float normSign = 1.0f;
    int bit = 1;
    for (int j = 0; j < 2; j++) {
        for (int i = 0; i != 3; ++i) {
            if ((so & bit) != 0) {
                float lambda = (-coord(source, i) - coord(he, i) * normSign) / coord(r, i);
                if (enter <= lambda) enter = lambda;
            } else if ((to_ & bit) != 0) {
                float lambda = (-coord(source, i) - coord(he, i) * normSign) / coord(r, i);
                exit = jmin(exit, lambda);
            }
            bit <<= 1;
        }
        normSign = -1.0f;
    }
    if (enter <= exit) { param = enter; return true; }
    return false;
}

// VectorUtil.setInterpolate3 (linearmath/VectorUtil.java:137-144)
static V3 interp3(V3 a, V3 b, float rt) {
    float s = 1.0f - rt;
    return v3(s * a.x + rt * b.x, s * a.y + rt * b.y, s * a.z + rt * b.z);
}

// SubsimplexConvexCast.calcTimeOfImpact (collision/narrowphase/SubsimplexConvexCast.java:62-191)
// for rayTestSingle's cast: A is a sphere of radius 0 (support: its centre) moving from the ray's
// start to its end with the identity basis, B the object's convex shape at rest.
static bool subsimplex_ray(const Shape& sb, const Xf& tB, V3 from, V3 to, float& fraction, V3& normal) {
    VoronoiSimplex s;
    s.reset();
    const V3 zero = v3(0.0f, 0.0f, 0.0f);
    Xf fromA = xf_identity(), toA = xf_identity();
    fromA.o = from;
    toA.o = to;
    V3 linVelA = sub(toA.o, fromA.o), linVelB = sub(tB.o, tB.o);
    float lambda = 0.0f;
    Xf iA = fromA, iB = tB;
    V3 r = sub(linVelA, linVelB);
    V3 supA = xf_apply(fromA, zero);
    V3 supB = xf_apply(tB, support_with_margin(sb, mulMTv(r, tB.b)));
    V3 v = sub(supA, supB);
    int maxIter = 32;
    V3 n = zero;
    float dist2 = len2(v);
    const float epsilon = 0.0001f;
    while ((dist2 > epsilon) && (maxIter--) != 0) {
        supA = xf_apply(iA, zero);
        supB = xf_apply(iB, support_with_margin(sb, mulMTv(v, iB.b)));
        V3 w = sub(supA, supB);
        float VdotW = dot(v, w);
        if (lambda > 1.0f) return false;
        if (VdotW > 0.0f) {
            float VdotR = dot(v, r);
            if (VdotR >= -(FLT_EPS * FLT_EPS)) return false;
            lambda = lambda - VdotW / VdotR;
            iA.o = interp3(fromA.o, toA.o, lambda);
            iB.o = interp3(tB.o, tB.o, lambda);
            w = sub(supA, supB);
            n = v;
        }
        s.addVertex(w, supA, supB);
        if (s.closest(v)) dist2 = len2(v);
        else dist2 = 0.0f;
    }
    fraction = lambda;
    normal = len2(n) >= FLT_EPS * FLT_EPS ? nor(n) : zero;
    if (dot(normal, r) >= -0.0f) return false;   // -allowedPenetration (0)
    return true;
}

namespace {
struct RayCallback {          // ClosestRayResultCallback
    float closest = 1.0f;
    int body = -1;
    V3 normal{0, 0, 0};
};
}  // namespace

// TriangleRaycastCallback.processTriangle (collision/narrowphase/TriangleRaycastCallback.java:
// 47-117) with BridgeTriangleRaycastCallback.reportHit (CollisionWorld.java:820-829).
static void ray_triangle(const V3 tri[3], V3 from, V3 to, float& hitFraction, int body, const Xf& objXf, RayCallback& cb) {
    V3 v10 = sub(tri[1], tri[0]), v20 = sub(tri[2], tri[0]);
    V3 tn = crs(v10, v20);
    float dist = dot(tri[0], tn);
    float dist_a = dot(tn, from) - dist;
    float dist_b = dot(tn, to) - dist;
    if (dist_a * dist_b >= 0.0f) return;
    float proj = dist_a - dist_b;
    float distance = dist_a / proj;
    if (!(distance < hitFraction)) return;
    float tol = len2(tn) * -0.0001f;
    V3 point = interp3(from, to, distance);
    V3 v0p = sub(tri[0], point), v1p = sub(tri[1], point);
    if (!(dot(crs(v0p, v1p), tn) >= tol)) return;
    V3 v2p = sub(tri[2], point);
    if (!(dot(crs(v1p, v2p), tn) >= tol)) return;
    if (!(dot(crs(v2p, v0p), tn) >= tol)) return;
    V3 nl = dist_a > 0.0f ? tn : scl(tn, -1.0f);
    cb.closest = distance;                        // ClosestRayResultCallback.addSingleResult
    cb.body = body;
    cb.normal = mulMv(nl, objXf.b);               // normal not in world space: times the basis
    hitFraction = distance;
}

// rayTestSingle's concave branch for a StaticPlaneShape: the ray in the object's space and
// StaticPlaneShape.processAllTriangles (collision/shapes/StaticPlaneShape.java:60-120), which
// spans two triangles around the ray's local aabb; the port takes half of the aabb's minimum
// corner as the half extent (halfExtents.set(aabbMax).set(aabbMin)).
static void ray_plane(const Shape& sh, const Xf& t, int body, V3 fromW, V3 toW, RayCallback& cb) {
    Xf inv = xf_inverse(t);
    V3 from = xf_apply(inv, fromW), to = xf_apply(inv, toW);
    float hitFraction = cb.closest;
    V3 mn = v3(jmin(from.x, to.x), jmin(from.y, to.y), jmin(from.z, to.z));
    V3 mx = v3(jmax(from.x, to.x), jmax(from.y, to.y), jmax(from.z, to.z));
    V3 half = scl(mn, 0.5f);
    float radius = len(half);
    V3 center = scl(add(mx, mn), 0.5f);
    V3 t0, t1;
    plane_space1(sh.planeNormal, t0, t1);
    V3 pc = sub(center, scl(sh.planeNormal, dot(sh.planeNormal, center) - sh.planeConstant));
    V3 a = scl(t0, radius), b = scl(t1, radius);
    V3 tri[3];
    tri[0] = add(add(pc, a), b);
    tri[1] = add(pc, sub(a, b));
    tri[2] = sub(pc, sub(a, b));
    ray_triangle(tri, from, to, hitFraction, body, t, cb);
    tri[0] = sub(pc, sub(a, b));
    tri[1] = sub(pc, add(a, b));
    tri[2] = add(add(pc, a), b);
    ray_triangle(tri, from, to, hitFraction, body, t, cb);
}

// OptimizedBvh.walkStacklessQuantizedTreeAgainstRay (OptimizedBvh.java:817-938): the leaves a ray
// (or a box cast: the box's extents aabbMin / aabbMax added to the ray's box and to every node's
// box) reaches, in walk order.  A node is entered when its quantized box overlaps the query's
// quantized box and AabbUtil2.rayAabb (bound 1) accepts its unquantized, widened box.
static void mesh_cast_walk(const MeshData& m, V3 from, V3 to, V3 bmin, V3 bmax, std::vector<int>& out) {
    out.clear();
    const QuantizedBvh& q = m.bvh;
    V3 amin = v3(jmin(from.x, to.x), jmin(from.y, to.y), jmin(from.z, to.z));
    V3 amax = v3(jmax(from.x, to.x), jmax(from.y, to.y), jmax(from.z, to.z));
    amin = add(amin, bmin);
    amax = add(amax, bmax);
    auto quant = [&](V3 p, int o[3]) {   // quantizeWithClamp
        V3 c = v3(jmax(p.x, q.bvhAabbMin.x), jmax(p.y, q.bvhAabbMin.y), jmax(p.z, q.bvhAabbMin.z));
        c = v3(jmin(c.x, q.bvhAabbMax.x), jmin(c.y, q.bvhAabbMax.y), jmin(c.z, q.bvhAabbMax.z));
        V3 v = mulc(sub(c, q.bvhAabbMin), q.bvhQuantization);
        o[0] = (int)(v.x + 0.5f) & 0xFFFF;
        o[1] = (int)(v.y + 0.5f) & 0xFFFF;
        o[2] = (int)(v.z + 0.5f) & 0xFFFF;
    };
    auto unquant = [&](const uint16_t* n) {
        V3 v = v3((float)n[0] / q.bvhQuantization.x, (float)n[1] / q.bvhQuantization.y, (float)n[2] / q.bvhQuantization.z);
        return add(v, q.bvhAabbMin);
    };
    int qa[3], qb[3];
    quant(amin, qa);
    quant(amax, qb);
    int cur = 0;
    while (cur < q.curNodeIndex) {
        const uint16_t* n = &q.q[6 * cur];
        bool boxOv = !(qa[0] > n[3] || qb[0] < n[0]) && !(qa[2] > n[5] || qb[2] < n[2]) && !(qa[1] > n[4] || qb[1] < n[1]);
        bool leaf = q.escOrTri[cur] >= 0;
        bool rayOv = false;
        if (boxOv) {
            V3 b0 = add(unquant(n), bmin), b1 = add(unquant(n + 3), bmax);
            float param = 1.0f;
            rayOv = ray_aabb(from, to, b0, b1, param);
        }
        if (leaf && rayOv) out.push_back(q.escOrTri[cur] & ((1 << 21) - 1));
        if (rayOv || leaf) cur++;
        else cur += -q.escOrTri[cur];
    }
}

// rayTestSingle's BvhTriangleMeshShape branch (CollisionWorld.java:297-311): the ray in the mesh's
// space, BvhTriangleMeshShape.performRaycast -> OptimizedBvh.reportRayOverlappingNodex (no box
// extents, java:999-1015), each leaf reached tested by TriangleRaycastCallback.
static void ray_mesh(const Shape& sh, const Xf& t, int body, V3 fromW, V3 toW, RayCallback& cb) {
    Xf inv = xf_inverse(t);
    V3 from = xf_apply(inv, fromW), to = xf_apply(inv, toW);
    float hitFraction = cb.closest;
    std::vector<int> tris;
    mesh_cast_walk(*sh.mesh, from, to, v3(0, 0, 0), v3(0, 0, 0), tris);
    for (int tri : tris) {
        V3 tv[3] = {sh.mesh->tri[3 * tri], sh.mesh->tri[3 * tri + 1], sh.mesh->tri[3 * tri + 2]};
        ray_triangle(tv, from, to, hitFraction, body, t, cb);
    }
}

// rayTestSingle's convex branch (CollisionWorld.java:267-293) on one convex shape at t.
static void ray_convex(const Shape& sh, const Xf& t, int body, V3 from, V3 to, RayCallback& cb) {
    float f;
    V3 n;
    if (subsimplex_ray(sh, t, from, to, f, n) && len2(n) > 0.0001f && f < cb.closest) {
        cb.closest = f;
        cb.body = body;
        cb.normal = nor(mulMv(n, m3_identity()));   // rotated by the ray's (identity) basis
    }
}

RayResult ray_test(const World& w, V3 from, V3 to, int group, int mask, int world) {
    RayCallback cb;
    for (size_t i = 0; i < w.bodies.size(); i++) {
        if (cb.closest == 0.0f) break;
        const Body& b = w.bodies[i];
        if (b.world != world) continue;
        if (((b.group & mask) & 0xFFFF) == 0 || ((group & b.mask) & 0xFFFF) == 0) continue;   // needsCollision
        const Shape& sh = w.shapes[b.shape];
        V3 mn, mx;
        shape_aabb(sh, b.xf, mn, mx);
        float param = cb.closest;
        if (!ray_aabb(from, to, mn, mx, param)) continue;
        if (sh.isConvex()) {
            ray_convex(sh, b.xf, (int)i, from, to, cb);
        } else if (sh.type == TRIANGLE_MESH) {
            ray_mesh(sh, b.xf, (int)i, from, to, cb);
        } else if (sh.isCompound()) {   // rayTestSingle's compound branch (CollisionWorld.java:340-355)
            for (size_t c = 0; c < sh.children.size(); c++)
                ray_convex(sh.children[c], xf_mul(b.xf, sh.childXf[c]), (int)i, from, to, cb);
        } else {
            ray_plane(sh, b.xf, (int)i, from, to, cb);
        }
    }
    RayResult r;
    r.body = cb.body;
    r.fraction = cb.closest;
    r.normal = cb.normal;
    r.point = cb.body >= 0 ? interp3(from, to, cb.closest) : v3(0.0f, 0.0f, 0.0f);
    return r;
}


// ----------------------------------------------------------------------------------------
// CollisionWorld.convexSweepTest with a ClosestConvexResultCallback (collision/dispatch/
// CollisionWorld.java:596-645, objectQuerySingle 391-490, ClosestConvexResultCallback 766-805)
// ----------------------------------------------------------------------------------------
// TransformUtil.calculateVelocity / calculateDiffAxisAngle (linearmath/TransformUtil.java:105-153)
void calculate_velocity(const Xf& t0, const Xf& t1, float timeStep, V3& linVel, V3& angVel) {
    linVel = scl(sub(t1.o, t0.o), 1.0f / timeStep);
    M3 dmat = mulMM(t1.b, m3_invert(t0.b));
    Quat dorn = qnor(q_from_matrix(dmat));
    float angle = 2.0f * jacos(dorn.w);                     // QuaternionUtil.getAngle
    V3 axis = v3(dorn.x, dorn.y, dorn.z);
    float l2 = len2(axis);
    if (l2 < FLT_EPS * FLT_EPS) axis = v3(1.0f, 0.0f, 0.0f);
    else axis = scl(axis, 1.0f / jsqrt(l2));
    angVel = scl(axis, angle / timeStep);
}

// CollisionShape.calculateTemporalAabb (collision/shapes/CollisionShape.java:76-121) with
// getAngularMotionDisc / getBoundingSphere (44-72).
void temporal_aabb(const Shape& s, const Xf& cur, V3 linvel, V3 angvel, float timeStep, V3& mn, V3& mx) {
    shape_aabb(s, cur, mn, mx);
    V3 lin = scl(linvel, timeStep);
    if (lin.x > 0.0f) mx.x += lin.x; else mn.x += lin.x;
    if (lin.y > 0.0f) mx.y += lin.y; else mn.y += lin.y;
    if (lin.z > 0.0f) mx.z += lin.z; else mn.z += lin.z;
    V3 bmin, bmax;
    shape_aabb(s, xf_identity(), bmin, bmax);
    float radius = len(sub(bmax, bmin)) * 0.5f;
    V3 center = scl(add(bmin, bmax), 0.5f);
    float disc = radius + len(center);
    float am = len(angvel) * disc * timeStep;
    mn = sub(mn, v3(am, am, am));
    mx = add(mx, v3(am, am, am));
}

// GjkConvexCast.calcTimeOfImpact (collision/narrowphase/GjkConvexCast.java:67-185): conservative
// advancement on GjkPairDetector distances (no penetration solver), through a PointCollector
// that keeps its closest result across the calls.
static bool gjk_convex_cast(const Shape& sa, const Xf& fromA, const Xf& toA, const Shape& sb, const Xf& tB,
                            float allowedPenetration, float& fraction, V3& normal, V3& hitPoint) {
    V3 r = sub(sub(toA.o, fromA.o), sub(tB.o, tB.o));
    const float radius = 0.001f;
    float lambda = 0.0f, lastLambda = 0.0f;
    int numIter = 0;
    bool has = false;
    float cdist = 1e30f;
    V3 cn = v3(0, 0, 0), cp = v3(0, 0, 0);
    auto collect = [&](const GjkOut& o) {
        if (o.valid && o.distance < cdist) { has = true; cn = o.normal; cp = o.pointOnB; cdist = o.distance; }
    };
    Xf iA = fromA, iB = tB;
    collect(gjk_closest_points(sa, iA, sb, iB, SIMD_INFINITY, false));
    if (!has) return false;
    V3 c = cp, n = cn;
    float dist = cdist;
    while (dist > radius) {
        if (++numIter > 32) return false;
        float dLambda = dist / dot(r, n);
        lambda = lambda - dLambda;
        if (lambda > 1.0f || lambda < 0.0f || lambda <= lastLambda) return false;
        lastLambda = lambda;
        iA.o = interp3(fromA.o, toA.o, lambda);
        iB.o = interp3(tB.o, tB.o, lambda);
        collect(gjk_closest_points(sa, iA, sb, iB, SIMD_INFINITY, false));
        if (cdist < 0.0f) { fraction = lastLambda; normal = cn; hitPoint = cp; return true; }
        c = cp;
        n = cn;
        dist = cdist;
    }
    if (dot(n, r) >= -allowedPenetration) return false;
    fraction = lambda;
    normal = n;
    hitPoint = c;
    return true;
}

// convexSweepTest over the bodies of one batch world.  The cast shape's temporal aabb comes from
// the sweep's start rotation; every object's aabb is grown by it and tested against the path of
// the origins with the bound 1 (not the closest hit so far), then GjkConvexCast.  A static plane
// reached by the sweep makes the reference throw (its plane branch calls a caster that is null):
// *planeHit is set and the result is that of the objects before it.
// SubsimplexConvexCast.calcTimeOfImpact (collision/narrowphase/SubsimplexConvexCast.java:62-191)
// for A moving from fromA to toA (origins interpolated, A's basis kept), B at rest at tB,
// allowedPenetration 0 (a fresh CastResult): the fraction, the unit normal and B's closest point.
static bool subsimplex_cast(const Shape& sa, const Xf& fromA, const Xf& toA, const Shape& sb, const Xf& tB,
                            float& fraction, V3& normal, V3& hitPoint) {
    VoronoiSimplex s;
    s.reset();
    const V3 zero = v3(0.0f, 0.0f, 0.0f);
    V3 linVelA = sub(toA.o, fromA.o), linVelB = sub(tB.o, tB.o);
    float lambda = 0.0f;
    Xf iA = fromA, iB = tB;
    V3 r = sub(linVelA, linVelB);
    V3 supA = xf_apply(fromA, support_with_margin(sa, mulMTv(scl(r, -1.0f), fromA.b)));
    V3 supB = xf_apply(tB, support_with_margin(sb, mulMTv(r, tB.b)));
    V3 v = sub(supA, supB);
    int maxIter = 32;
    V3 n = zero;
    float dist2 = len2(v);
    while ((dist2 > 0.0001f) && (maxIter--) != 0) {
        supA = xf_apply(iA, support_with_margin(sa, mulMTv(scl(v, -1.0f), iA.b)));
        supB = xf_apply(iB, support_with_margin(sb, mulMTv(v, iB.b)));
        V3 w = sub(supA, supB);
        float VdotW = dot(v, w);
        if (lambda > 1.0f) return false;
        if (VdotW > 0.0f) {
            float VdotR = dot(v, r);
            if (VdotR >= -(FLT_EPS * FLT_EPS)) return false;
            lambda = lambda - VdotW / VdotR;
            iA.o = interp3(fromA.o, toA.o, lambda);
            iB.o = interp3(tB.o, tB.o, lambda);
            w = sub(supA, supB);
            n = v;
        }
        s.addVertex(w, supA, supB);
        if (s.closest(v)) dist2 = len2(v);
        else dist2 = 0.0f;
    }
    fraction = lambda;
    normal = len2(n) >= FLT_EPS * FLT_EPS ? nor(n) : zero;
    if (dot(normal, r) >= -0.0f) return false;
    V3 hA, hB;
    s.compute_points(hA, hB);
    hitPoint = hB;
    return true;
}

// objectQuerySingle's BvhTriangleMeshShape branch (CollisionWorld.java:425-455): the cast's
// origins in the mesh's space and its shape's aabb at the mesh-space rotation of its end
// transform widen the ray of BvhTriangleMeshShape.performConvexcast
// (OptimizedBvh.reportBoxCastOverlappingNodex, java:1017-1036); each triangle reached is cast
// against by TriangleConvexcastCallback.processTriangle (TriangleConvexcastCallback.java:53-88:
// SubsimplexConvexCast, the fraction below the callback's hitFraction - which it never lowers -,
// the normal normalised once more) and reported through BridgeTriangleConvexcastCallback.reportHit
// (CollisionWorld.java:840-851: accepted when the fraction is <= the result callback's closest).
// accept(f, n, p) stands for the result callback's addSingleResult and returns its closest.
template <class Accept>
static void sweep_mesh(const Shape& cast, const Xf& from, const Xf& to, const Shape& mesh, const Xf& tM, float closest,
                       Accept accept) {
    Xf inv = xf_inverse(tM);
    V3 fromL = xf_apply(inv, from.o), toL = xf_apply(inv, to.o);
    Xf rot;
    rot.b = mulMM(inv.b, to.b);   // rotationXform.set(worldToObject.basis * convexToTrans.basis)
    rot.o = v3(0.0f, 0.0f, 0.0f);
    V3 bmin, bmax;
    shape_aabb(cast, rot, bmin, bmax);
    std::vector<int> tris;
    mesh_cast_walk(*mesh.mesh, fromL, toL, bmin, bmax, tris);
    const float hitFraction = closest;
    Shape tm;
    tm.type = TRIANGLE;
    tm.collisionMargin = mesh.getMargin();
    for (int t : tris) {
        for (int k = 0; k < 3; k++) tm.tri[k] = mesh.mesh->tri[3 * t + k];
        float f;
        V3 n, p;
        if (!subsimplex_cast(cast, from, to, tm, tM, f, n, p)) continue;
        if (!(len2(n) > 0.0001f) || !(f < hitFraction)) continue;
        n = nor(n);
        if (f <= closest) closest = accept(f, n, p);
    }
}

RayResult convex_sweep(const World& w, const Shape& cast, const Xf& from, const Xf& to, int group, int mask, int world,
                       bool* planeHit) {
    *planeHit = false;
    V3 linVel, angVel;
    calculate_velocity(from, to, 1.0f, linVel, angVel);
    Xf R = xf_identity();
    R.b = m3_from_quat(q_from_matrix(from.b));
    V3 cmin, cmax;
    temporal_aabb(cast, R, linVel, angVel, 1.0f, cmin, cmax);
    RayResult res;
    float closest = 1.0f;
    for (size_t i = 0; i < w.bodies.size(); i++) {
        const Body& b = w.bodies[i];
        if (b.world != world) continue;
        if (((b.group & mask) & 0xFFFF) == 0 || ((group & b.mask) & 0xFFFF) == 0) continue;
        const Shape& sh = w.shapes[b.shape];
        V3 mn, mx;
        shape_aabb(sh, b.xf, mn, mx);
        mn = add(mn, cmin);
        mx = add(mx, cmax);
        float param = 1.0f;
        if (!ray_aabb(from.o, to.o, mn, mx, param)) continue;
        if (sh.type == TRIANGLE_MESH) {
            sweep_mesh(cast, from, to, sh, b.xf, closest, [&](float f, V3 n, V3 p) {
                closest = f;   // ClosestConvexResultCallback.addSingleResult
                res.body = (int)i;
                res.fraction = f;
                res.normal = n;
                res.point = p;
                return closest;
            });
            continue;
        }
        if (!sh.isConvex() && !sh.isCompound()) { *planeHit = true; return res; }
        // objectQuerySingle's convex branch, or its compound branch over the children at the
        // body's transform times the child's (CollisionWorld.java:391-430, 491-510)
        const int nc = sh.isCompound() ? (int)sh.children.size() : 1;
        for (int c = 0; c < nc; c++) {
            const Shape& cs = sh.isCompound() ? sh.children[c] : sh;
            const Xf cx = sh.isCompound() ? xf_mul(b.xf, sh.childXf[c]) : b.xf;
            float f;
            V3 n, p;
            if (gjk_convex_cast(cast, from, to, cs, cx, 0.04f, f, n, p) && len2(n) > 0.0001f && f < closest) {
                closest = f;
                res.body = (int)i;
                res.fraction = f;
                res.normal = nor(n);
                res.point = p;
            }
        }
    }
    return res;
}

// The CCD sweep of integrateTransforms (dynamics/DiscreteDynamicsWorld.java:700-729): a sphere of
// the body's ccdSweptSphereRadius swept by convexSweepTest (CollisionWorld.java:596-645) from the
// body's transform to its predicted one, with ClosestNotMeConvexResultCallback (java:1129-1198).
// Objects are seen at their transforms of the moment: the bodies before `me` in the world's order
// have already been moved by this integrateTransforms.  needsCollision: not `me`, the proxies'
// filters, and, since every body here has contact response, HashedOverlappingPairCache.findPair
// (collision/broadphase/HashedOverlappingPairCache.java:231-265) - whose argument swap is broken
// (233-237), so it finds the pair only when `me` precedes the other object; a pair found with a
// manifold that holds contact points excludes the object.  addSingleResult drops hits whose
// normal does not oppose the motion (normal . (to - from) >= 0).  A static plane reached by the
// sweep makes the reference throw (objectQuerySingle's concave branch, CollisionWorld.java:
// 470-490): *planeHit is set and the plane is skipped.
bool ccd_sweep(const World& w, int me, const Xf& to, float& fraction, bool* planeHit) {
    *planeHit = false;
    const Body& mb = w.bodies[me];
    const Xf from = mb.xf;
    const Shape cast = make_sphere(mb.ccdSweptSphereRadius);
    V3 linVel, angVel;
    calculate_velocity(from, to, 1.0f, linVel, angVel);
    Xf R = xf_identity();
    R.b = m3_from_quat(q_from_matrix(from.b));
    V3 cmin, cmax;
    temporal_aabb(cast, R, linVel, angVel, 1.0f, cmin, cmax);
    const V3 motion = sub(to.o, from.o);        // the callback's convexToWorld - convexFromWorld
    float closest = 1.0f;
    bool hit = false;
    for (size_t i = 0; i < w.bodies.size(); i++) {
        const Body& b = w.bodies[i];
        if ((int)i == me || b.world != mb.world) continue;
        if (((b.group & mb.mask) & 0xFFFF) == 0 || ((mb.group & b.mask) & 0xFFFF) == 0) continue;
        if (mb.hasContactResponse() && b.hasContactResponse() && me < (int)i) {
            // the pair's algorithm's manifolds (getAllContactManifolds): one per child combination
            bool touching = false;
            for (int sub = 0, ns = pair_subs(w, me, (int)i); sub < ns && !touching; sub++) {
                const uint64_t key = pair_key(w, me, (int)i) | ((uint64_t)sub << 24);
                auto it = std::lower_bound(w.pairKeys.begin(), w.pairKeys.end(), key);
                if (it != w.pairKeys.end() && *it == key) {
                    const size_t k = (size_t)(it - w.pairKeys.begin());
                    touching = w.pairHasAlgo[k] && w.pairMf[k].n > 0;
                }
            }
            if (touching) continue;
        }
        const Shape& sh = w.shapes[b.shape];
        V3 mn, mx;
        shape_aabb(sh, b.xf, mn, mx);
        mn = add(mn, cmin);
        mx = add(mx, cmax);
        float param = 1.0f;
        if (!ray_aabb(from.o, to.o, mn, mx, param)) continue;
        if (sh.type == TRIANGLE_MESH) {
            sweep_mesh(cast, from, to, sh, b.xf, closest, [&](float f, V3 n, V3) {
                if (dot(n, motion) >= -0.0f) return closest;   // ClosestNotMeConvexResultCallback rejects
                closest = f;
                hit = true;
                return closest;
            });
            continue;
        }
        if (!sh.isConvex() && !sh.isCompound()) { *planeHit = true; continue; }
        const int nc = sh.isCompound() ? (int)sh.children.size() : 1;
        for (int c = 0; c < nc; c++) {
            const Shape& cs = sh.isCompound() ? sh.children[c] : sh;
            const Xf cx = sh.isCompound() ? xf_mul(b.xf, sh.childXf[c]) : b.xf;
            float f;
            V3 n, p;
            if (gjk_convex_cast(cast, from, to, cs, cx, 0.04f, f, n, p) && len2(n) > 0.0001f && f < closest) {
                if (dot(nor(n), motion) >= -0.0f) continue;   // moving away from the contact normal
                closest = f;
                hit = true;
            }
        }
    }
    fraction = closest;
    return hit;
}

}  // namespace jb
