// Triangle-mesh shapes on the host: the quantized tree and local aabb of a
// BvhTriangleMeshShape (meshes.cu).
#pragma once
#include <cmath>
#include <utility>
#include <vector>
#include <cuda_runtime.h>

namespace jbg {

struct MeshBvh {
    std::vector<float4> tris;   // 3 vertices per triangle, by triangle index
    std::vector<int4> nodes;    // quantized nodes in walk order (layout: DevShapes::mesh_nodes)
    float bmin[3], bmax[3], quant[3];
    float lmin[3], lmax[3];     // TriangleMeshShape.localAabbMin / Max (margin 0)
};

// Returns nonzero for an empty mesh, an index out of range or more than 2^21 - 1 triangles.
int build_mesh_bvh(const float* vertices, int numVertices, const int* indices, int numTriangles, MeshBvh& out);

// BvhTriangleMeshShape.refitTree over new vertex positions: m holds the tree built over the same
// indices; its triangles, quantization, node boxes and local aabb (with the shape's current
// margin) are updated, its topology kept.
void refit_mesh_bvh(const float* vertices, const int* indices, int numTriangles, float margin, MeshBvh& m);

}  // namespace jbg
