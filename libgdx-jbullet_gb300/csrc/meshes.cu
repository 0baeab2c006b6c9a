// Host side of the triangle-mesh shape: BvhTriangleMeshShape's quantized OptimizedBvh, built
// once when the shape is added, as the reference's constructor builds it
// (collision/shapes/BvhTriangleMeshShape.java:69-93, OptimizedBvh.java:128-342,480-707), and the
// mesh's local aabb (TriangleMeshShape.recalcLocalAabb, TriangleMeshShape.java:79-95).
//
// The node order decides the order in which a query reports overlapping triangles, and so the
// order in which their contact points reach a manifold; the tree is therefore rebuilt here with
// the reference's splitting rule and its binary32 arithmetic (host code is compiled without
// floating-point contraction), node for node.  The nodes are written depth first, left subtree
// first, from an explicit work stack.
#include <cstdint>
#include <vector>

#include "meshes.cuh"

namespace jbg {
namespace {

// java.lang.Math.max / min on floats (NaN first, -0 below +0)
float fmax_j(float a, float b) {
    if (a != a) return a;
    if (a == 0.0f && b == 0.0f) return std::signbit(a) ? b : a;
    return a >= b ? a : b;
}
float fmin_j(float a, float b) {
    if (a != a) return a;
    if (a == 0.0f && b == 0.0f) return std::signbit(b) ? b : a;
    return a <= b ? a : b;
}

struct Builder {
    float bmin[3], bmax[3], quant[3];
    std::vector<uint16_t> leaf;        // 6 per leaf: quantized min xyz, max xyz
    std::vector<int> leafTri;
    std::vector<uint16_t> node;        // 6 per node
    std::vector<int> nodeW;            // triangle index (leaf) or -escapeIndex

    void quantize(const float p[3], uint16_t out[3]) const {   // OptimizedBvh.quantizeWithClamp
        for (int k = 0; k < 3; k++) {
            float c = fmin_j(fmax_j(p[k], bmin[k]), bmax[k]);
            float v = (c - bmin[k]) * quant[k];
            out[k] = (uint16_t)((int)(v + 0.5f) & 0xFFFF);
        }
    }
    void unquantize(const uint16_t* q, float out[3]) const {    // OptimizedBvh.unQuantize
        for (int k = 0; k < 3; k++) out[k] = (float)q[k] / quant[k] + bmin[k];
    }
    void centre(int i, float c[3]) const {
        float mn[3], mx[3];
        unquantize(&leaf[6 * i], mn);
        unquantize(&leaf[6 * i + 3], mx);
        for (int k = 0; k < 3; k++) c[k] = (mx[k] + mn[k]) * 0.5f;
    }
    void means(int a, int b, float m[3]) const {
        m[0] = m[1] = m[2] = 0.0f;
        for (int i = a; i < b; i++) {
            float c[3];
            centre(i, c);
            for (int k = 0; k < 3; k++) m[k] = m[k] + c[k];
        }
        const float inv = 1.0f / (float)(b - a);
        for (int k = 0; k < 3; k++) m[k] = m[k] * inv;
    }
    int split_axis(int a, int b) const {                         // OptimizedBvh.calcSplittingAxis
        float m[3], var[3] = {0.0f, 0.0f, 0.0f};
        means(a, b, m);
        for (int i = a; i < b; i++) {
            float c[3];
            centre(i, c);
            for (int k = 0; k < 3; k++) {
                float d = c[k] - m[k];
                var[k] = var[k] + d * d;
            }
        }
        const float inv = 1.0f / ((float)(b - a) - 1.0f);
        int axis = -1;
        float best = -1e30f;
        for (int k = 0; k < 3; k++) {
            float v = var[k] * inv;
            if (v > best) { best = v; axis = k; }
        }
        return axis < 0 ? 2 : axis;   // VectorUtil.getCoord reads z for an index out of range
    }
    int split_index(int a, int b, int axis) {                    // OptimizedBvh.sortAndCalcSplittingIndex
        float m[3];
        means(a, b, m);
        int split = a;
        for (int i = a; i < b; i++) {
            float c[3];
            centre(i, c);
            if (c[axis] > m[axis]) {
                for (int k = 0; k < 6; k++) std::swap(leaf[6 * i + k], leaf[6 * split + k]);
                std::swap(leafTri[i], leafTri[split]);
                split++;
            }
        }
        const int n = b - a, third = n / 3;
        if (split <= a + third || split >= b - 1 - third) split = a + (n >> 1);
        return split;
    }
    // OptimizedBvh.buildTree: a range of one leaf becomes that leaf's node; a larger range an
    // internal node (its box the quantized union of its leaves' boxes) followed by its left and
    // right subtrees, its escape index the node count of its subtree.
    void build(int nLeaves) {
        node.assign((size_t)12 * nLeaves, 0);
        nodeW.assign((size_t)2 * nLeaves, 0);
        struct Task { int a, b, close; };   // close >= 0: set that node's escape index
        std::vector<Task> stack{{0, nLeaves, -1}};
        int cur = 0;
        while (!stack.empty()) {
            Task t = stack.back();
            stack.pop_back();
            if (t.close >= 0) {
                nodeW[t.close] = -(cur - t.close);
                continue;
            }
            if (t.b - t.a == 1) {
                for (int k = 0; k < 6; k++) node[6 * cur + k] = leaf[6 * t.a + k];
                nodeW[cur] = leafTri[t.a];
                cur++;
                continue;
            }
            const int axis = split_axis(t.a, t.b);
            const int split = split_index(t.a, t.b, axis);
            const int id = cur++;
            const float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
            quantize(lo, &node[6 * id]);
            quantize(hi, &node[6 * id + 3]);
            for (int i = t.a; i < t.b; i++) {
                float mn[3], mx[3];
                uint16_t qa[3], qb[3];
                unquantize(&leaf[6 * i], mn);
                unquantize(&leaf[6 * i + 3], mx);
                quantize(mn, qa);
                quantize(mx, qb);
                for (int k = 0; k < 3; k++) {
                    if (node[6 * id + k] > qa[k]) node[6 * id + k] = qa[k];
                    if (node[6 * id + 3 + k] < qb[k]) node[6 * id + 3 + k] = qb[k];
                }
            }
            stack.push_back({0, 0, id});
            stack.push_back({split, t.b, -1});
            stack.push_back({t.a, split, -1});
        }
        node.resize((size_t)6 * cur);
        nodeW.resize(cur);
    }
};

// TriangleMeshShape.recalcLocalAabb (TriangleMeshShape.java:79-95): per axis the first vertex, in
// walk order (every leaf), with the largest (smallest) coordinate, taken through the dot with the
// unit axis as the support callback does, plus (minus) the shape's margin at that time.
void local_aabb(MeshBvh& m, float margin) {
    const int nn = (int)m.nodes.size();
    for (int k = 0; k < 3; k++) {
        for (int sg = 0; sg < 2; sg++) {
            float dir[3] = {0.0f, 0.0f, 0.0f};
            dir[k] = sg == 0 ? 1.0f : -1.0f;
            float best = -1e30f, sup = 0.0f;
            for (int i = 0; i < nn; i++) {
                if (m.nodes[i].w < 0) continue;
                for (int j = 0; j < 3; j++) {
                    const float4& p = m.tris[3 * (m.nodes[i].w & ((1 << 21) - 1)) + j];
                    const float d = dir[0] * p.x + dir[1] * p.y + dir[2] * p.z;
                    if (d > best) { best = d; sup = k == 0 ? p.x : (k == 1 ? p.y : p.z); }
                }
            }
            if (sg == 0) m.lmax[k] = sup + margin;
            else m.lmin[k] = sup - margin;
        }
    }
}

}  // namespace

int build_mesh_bvh(const float* v, int nv, const int* idx, int nt, MeshBvh& out) {
    if (!v || !idx || nv <= 0 || nt <= 0 || nt >= (1 << 21)) return 1;
    for (int i = 0; i < 3 * nt; i++)
        if (idx[i] < 0 || idx[i] >= nv) return 1;
    out.tris.resize((size_t)3 * nt);
    for (int i = 0; i < nt; i++)
        for (int k = 0; k < 3; k++) {
            const float* p = v + 3 * idx[3 * i + k];
            out.tris[3 * i + k] = make_float4(p[0], p[1], p[2], 0.0f);
        }
    // StridingMeshInterface.calculateAabbBruteForce, then setQuantizationValues(min, max, 1)
    float amin[3] = {1e30f, 1e30f, 1e30f}, amax[3] = {-1e30f, -1e30f, -1e30f};
    for (const float4& p : out.tris) {
        const float c[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; k++) { amin[k] = fmin_j(amin[k], c[k]); amax[k] = fmax_j(amax[k], c[k]); }
    }
    Builder b;
    for (int k = 0; k < 3; k++) {
        b.bmin[k] = amin[k] - 1.0f;
        b.bmax[k] = amax[k] + 1.0f;
        b.quant[k] = 65535.0f / (b.bmax[k] - b.bmin[k]);
    }
    // QuantizedNodeTriangleCallback: a leaf per triangle, its box widened to 0.002 where thinner
    b.leaf.resize((size_t)6 * nt);
    b.leafTri.resize(nt);
    for (int i = 0; i < nt; i++) {
        float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
        for (int j = 0; j < 3; j++) {
            const float4& p = out.tris[3 * i + j];
            const float c[3] = {p.x, p.y, p.z};
            for (int k = 0; k < 3; k++) { mn[k] = fmin_j(mn[k], c[k]); mx[k] = fmax_j(mx[k], c[k]); }
        }
        for (int k = 0; k < 3; k++)
            if (mx[k] - mn[k] < 0.002f) {
                mx[k] = mx[k] + 0.001f;
                mn[k] = mn[k] - 0.001f;
            }
        b.quantize(mn, &b.leaf[6 * i]);
        b.quantize(mx, &b.leaf[6 * i + 3]);
        b.leafTri[i] = i;   // part 0
    }
    b.build(nt);
    const int nn = (int)b.nodeW.size();
    out.nodes.resize(nn);
    for (int i = 0; i < nn; i++) {
        const uint16_t* q = &b.node[6 * i];
        out.nodes[i] = make_int4((int)((unsigned)q[0] | ((unsigned)q[1] << 16)), (int)((unsigned)q[2] | ((unsigned)q[3] << 16)),
                                 (int)((unsigned)q[4] | ((unsigned)q[5] << 16)), b.nodeW[i]);
    }
    for (int k = 0; k < 3; k++) { out.bmin[k] = b.bmin[k]; out.bmax[k] = b.bmax[k]; out.quant[k] = b.quant[k]; }
    local_aabb(out, 0.0f);   // the shape's margin is 0 when the constructor runs
    return 0;
}

// OptimizedBvh.refit (OptimizedBvh.java:344-367): the quantization from the new brute-force box;
// updateBvhNodes (java:411-470) from the last node to the first: a leaf's box from its triangle
// (without the build's minimum extent), an internal node's the union of its two children's
// quantized boxes (the right child follows the left one's subtree); then recalcLocalAabb with
// the current margin (BvhTriangleMeshShape.refitTree, java:172-178).
void refit_mesh_bvh(const float* v, const int* idx, int nt, float margin, MeshBvh& m) {
    for (int i = 0; i < nt; i++)
        for (int k = 0; k < 3; k++) {
            const float* p = v + 3 * idx[3 * i + k];
            m.tris[3 * i + k] = make_float4(p[0], p[1], p[2], 0.0f);
        }
    float amin[3] = {1e30f, 1e30f, 1e30f}, amax[3] = {-1e30f, -1e30f, -1e30f};
    for (const float4& p : m.tris) {
        const float c[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; k++) { amin[k] = fmin_j(amin[k], c[k]); amax[k] = fmax_j(amax[k], c[k]); }
    }
    Builder b;
    for (int k = 0; k < 3; k++) {
        b.bmin[k] = amin[k] - 1.0f;
        b.bmax[k] = amax[k] + 1.0f;
        b.quant[k] = 65535.0f / (b.bmax[k] - b.bmin[k]);
        m.bmin[k] = b.bmin[k]; m.bmax[k] = b.bmax[k]; m.quant[k] = b.quant[k];
    }
    const int nn = (int)m.nodes.size();
    std::vector<uint16_t> q((size_t)6 * nn);
    for (int i = nn - 1; i >= 0; i--) {
        const int w = m.nodes[i].w;
        if (w >= 0) {
            float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
            for (int j = 0; j < 3; j++) {
                const float4& p = m.tris[3 * (w & ((1 << 21) - 1)) + j];
                const float c[3] = {p.x, p.y, p.z};
                for (int k = 0; k < 3; k++) { mn[k] = fmin_j(mn[k], c[k]); mx[k] = fmax_j(mx[k], c[k]); }
            }
            b.quantize(mn, &q[6 * i]);
            b.quantize(mx, &q[6 * i + 3]);
        } else {
            const int l = i + 1, r = m.nodes[l].w >= 0 ? i + 2 : i + 1 - m.nodes[l].w;
            for (int k = 0; k < 3; k++) {
                q[6 * i + k] = q[6 * l + k] > q[6 * r + k] ? q[6 * r + k] : q[6 * l + k];
                q[6 * i + 3 + k] = q[6 * l + 3 + k] < q[6 * r + 3 + k] ? q[6 * r + 3 + k] : q[6 * l + 3 + k];
            }
        }
    }
    for (int i = 0; i < nn; i++) {
        const uint16_t* p = &q[6 * i];
        m.nodes[i] = make_int4((int)((unsigned)p[0] | ((unsigned)p[1] << 16)), (int)((unsigned)p[2] | ((unsigned)p[3] << 16)),
                               (int)((unsigned)p[4] | ((unsigned)p[5] << 16)), m.nodes[i].w);
    }
    local_aabb(m, margin);
}

}  // namespace jbg
