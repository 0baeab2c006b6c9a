// Scene queries: CollisionWorld.rayTest with a ClosestRayResultCallback for batches of rays
// (collision/dispatch/CollisionWorld.java:553-591, rayTestSingle 260-331).
#pragma once
#include "../../include/jbgpu.h"
#include "broadphase.cuh"

namespace jbg {

struct QueryBuffers {
    float4* qmin = nullptr;       // per body: CollisionShape.getAabb at the current transform
    float4* qmax = nullptr;
    int capBodies = 0;
    float4* node = nullptr;       // the broadphase tree's topology refit over qmin / qmax
    int* visit = nullptr;
    int capNodes = 0;
    int* slow = nullptr;          // rays the closest-hit shortcut cannot decide (replayed in body order)
    int* slowCount = nullptr;
    int* rayCnt = nullptr;        // per ray: candidates, their offsets, the smallest hit key,
    int* rayOff = nullptr;        // the aabb entry of that hit's object, undecided flag
    unsigned long long* key = nullptr;
    float* enterJ = nullptr;
    int* undecided = nullptr;
    void* scanScratch = nullptr;
    int* candTotal = nullptr;
    unsigned long long* candTotal64 = nullptr;   // the same total in 64 bits (refuses overflowing batches)
    int capRays = 0;
    void* cand = nullptr;         // (ray, body, aabb entry) candidates and their hits
    float4* hitA = nullptr;
    float4* hitB = nullptr;
    int capCand = 0;
    int replayAll = 0;            // verification: every ray takes the in-order replay
    float* from = nullptr;        // staging for host buffers
    float* to = nullptr;
    int* rayWorld = nullptr;
    jbgpu_ray_hit* hits = nullptr;
    int capIo = 0;
    float4* sweepMin = nullptr;   // per sweep: the cast shape's temporal aabb, static plane on the
    float4* sweepMax = nullptr;   // path, the path of the origins (3 floats each)
    int* sweepPlane = nullptr;
    float* sweepFrom = nullptr;
    float* sweepTo = nullptr;
    int capSweeps = 0;
};

// Query boxes for every body and the refit tree over them; builds the broadphase tree first
// when the body set changed since its last build.
int query_prepare(const DevWorld& w, BroadphaseBuffers& bb, QueryBuffers& qb, cudaStream_t s);
// n rays (device buffers) against the prepared boxes; grows the replay list to n.  sms: blocks
// of the replay kernel.
int query_rays(const DevWorld& w, const BroadphaseBuffers& bb, QueryBuffers& qb, const float* from, const float* to,
               const int* rayWorld, int n, int group, int mask, jbgpu_ray_hit* hits, int sms, cudaStream_t s);
// n convex sweeps of shape `shape` (device buffers: 12-float transforms from / to, optional
// per-sweep batch world) against the prepared boxes and tree.  A sweep that reaches a static
// plane gets body -2.
int query_sweeps(const DevWorld& w, const BroadphaseBuffers& bb, QueryBuffers& qb, int shape, const float* from,
                 const float* to, const int* sweepWorld, int n, int group, int mask, jbgpu_ray_hit* hits, int sms,
                 cudaStream_t s);
void query_free(QueryBuffers& qb);

// CCD motion clamping of integrateTransforms (dynamics/DiscreteDynamicsWorld.java:679-739).
struct CcdBuffers {
    float4* pred = nullptr;       // per body: predicted transform, 3 float4 (basis rows, origin in .w)
    int* flag = nullptr;          // per body: runs a CCD sweep
    int* pos = nullptr;           // exclusive scan of flag
    int* list = nullptr;          // CCD bodies in index order
    void* scanScratch = nullptr;
    int cap = 0;
    int grid = 0;                 // co-resident blocks of the cooperative sweep kernel
};
// The integrate stage with CCD: predicted transforms, the CCD bodies' sweeps in index order (one
// cooperative launch, two grid barriers per CCD body), then every moved body's transform and
// world inverse inertia.  P / nPairs / cntp: the step's pair arrays (cntp nullable: nPairs exact).
int ccd_integrate(const DevWorld& w, const DevPairs& P, int nPairs, const int* cntp, CcdBuffers& cb, float dt, int sms,
                  cudaStream_t s);
// Buffers for n bodies and the sweep kernel's grid, ahead of a captured step (no allocation
// may happen while a stream is captured).
int ccd_reserve(CcdBuffers& cb, int n, int sms);
void ccd_free(CcdBuffers& cb);

}  // namespace jbg
