// Host side of the C ABI (include/jbgpu.h): world creation, body/shape upload, device
// buffer management and the per-step launch sequence of internalSingleStepSimulation
// (dynamics/DiscreteDynamicsWorld.java:356-400 of the reference):
//   predict -> aabbs -> pairs (count | host capacity check | fill, sort, persist)
//   -> narrowphase (GJK pass, EPA pass) -> islands -> colour + setup + PGS -> integrate
//   -> activation.
// All kernels of a world run on the world's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/jbgpu.h"
#include "broadphase.cuh"
#include "jbgpu_internal.cuh"
#include "mlp.cuh"
#include "narrowphase.cuh"
#include "meshes.cuh"
#include "prims.cuh"
#include "query.cuh"
#include "solver.cuh"

using namespace jbg;

// Kernel: CollisionWorld.updateSingleAabb for every body whose shape is `shape` (after a refit).
__global__ void k_shape_aabbs(DevWorld w, int shape);

static thread_local std::string g_err;
static int fail(int code, const std::string& msg) { g_err = msg; return code; }
namespace jbg {
int set_last_error(int code, const char* msg) { return fail(code, msg); }
}

#include <atomic>
static std::atomic<long long> g_launches{0};
void jbg::note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return fail(JBGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace {

// A triangle mesh's vertex count, triangle indices and scaling, kept for jbgpu_world_refit_mesh.
struct MeshSource {
    int shape = -1, numPoints = 0;
    std::vector<int> idx;
    float scaling[3] = {0.0f, 0.0f, 0.0f};
};

struct HostShape {
    int type;
    float margin;
    float dims[4];
    float lmin[4], lmax[4];
    float plane[4];
    int hull_off, hull_cnt;
    int child_off, child_cnt;          // compound: its children in jbgpu_world::childShapes / childXf
    int node_off, node_cnt, tri_off;   // triangle mesh: its tree nodes and triangles
    float q[12];                       // triangle mesh: bvhAabbMin, bvhAabbMax, bvhQuantization (xyz_)
};

template <class T> static cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc((void**)p, sizeof(T) * n);
}
template <class T> static void dfree(T*& p) { if (p) cudaFree((void*)p); p = nullptr; }

// Grow a device array to n elements keeping the first keep elements.
template <class T> static cudaError_t dgrow(T** p, size_t oldn, size_t n, size_t keep, cudaStream_t s) {
    T* q = nullptr;
    cudaError_t e = dalloc(&q, n);
    if (e != cudaSuccess) return e;
    if (*p && keep) e = cudaMemcpyAsync(q, *p, sizeof(T) * std::min(keep, oldn), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    cudaStreamSynchronize(s);
    if (*p) cudaFree(*p);
    *p = q;
    return cudaSuccess;
}

}  // namespace

struct jbgpu_world {
    jbgpu_config cfg;
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t aux = nullptr;       // second stream: island unions beside the narrowphase
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    cudaEvent_t evT0 = nullptr, evT1 = nullptr;   // jbgpu_world_timer
    float localTime = 1.0f / 60.0f;
    long long steps = 0;
    jbgpu_tick_callback tickCb = nullptr;   // DynamicsWorld.setInternalTickCallback
    void* tickUser = nullptr;
    bool inTick = false;
    // shapes
    std::vector<HostShape> shapes;
    std::vector<float4> hullPts;
    std::vector<HostShape> childShapes;   // compound children, appended after the shapes on the device
    std::vector<float4> childXf;          // 3 per child: basis rows, origin in .w
    std::vector<MeshSource> meshSrc;      // per triangle mesh: what a refit needs
    std::vector<int> aabbRefresh;         // shapes whose bodies' aabbs the next prepare recomputes
    std::vector<int4> meshNodes;          // quantized tree nodes of every triangle mesh
    std::vector<float4> meshTris;         // 3 vertices per triangle
    bool hasMesh = false, hasCompound = false;
    bool hasKinematic = false;            // some body is kinematic: saveKinematicState runs
    int candBound = 0;                    // the concave pass's candidates of this step (count pass bound)
    bool shapesDirty = true;
    int capShapes = 0, capHull = 0;
    // bodies
    int nBodies = 0, capBodies = 0;
    std::vector<int> hShape, hWorld, hFlags;
    int nWorlds = 1;
    bool planesDirty = true;
    std::vector<int> worldFinite;   // finite (non-plane) bodies per batch world
    // point-to-point joints (host copy; uploaded to sb.J when they change)
    std::vector<int> jKind, jA, jB;
    std::vector<float4> jPivA, jPivB, jSet, jSet2, jFrame;   // jFrame: 6 per joint
    std::vector<float4> jD6;                                  // D6_SET_F4 per joint
    bool jointsDirty = false;
    int capJoints = 0;
    bool orderValid = false;        // the broadphase leaf order covers every body added
    bool solverDirty = true;        // solver parts must be planned again
    int solverOrderFinite = -1;     // nFinite the parts were planned for
    DevWorld dw{};
    // pairs: two buffers, cur holds the pairs of the last broadphase
    DevPairs pairs[2]{};
    int capPairs[2] = {0, 0};
    int cur = 0;
    int nPairs = 0;
    int capRows = 0;          // pair-capacity of the pair-sized work buffers
    DevRows rows{};
    BroadphaseBuffers bb;
    NarrowBuffers nb;
    SolverBuffers sb;
    QueryBuffers qb;                  // ray queries
    CcdBuffers cb;                    // CCD motion clamping (jbgpu_world_set_ccd)
    bool ccdOn = false;               // some body has a CCD motion threshold
    const int* pairCountDev = nullptr;   // while the step's second graph is captured: the pair count
                                         // on the device (nPairs then being the capacity)
    int* hostPinned = nullptr;
    Prof prof;
    int* profHist = nullptr;      // per profiled step: device counters + solver manifolds
    float* ioStage = nullptr;     // device staging for apply_forces / get_transforms (12 floats per body)
    int capIo = 0;
    // learned warm start and training samples
    jbgpu_mlp* mlp = nullptr;     // not owned
    bool learnReady = false;      // warm-start kernel configured
    bool logSamples = false;
    bool logAll = false;          // samples of every point, not only of converged islands
    float* sampleX = nullptr;     // capRows * 4 * 24
    float* sampleT = nullptr;     // capRows * 4 * 3
    int sampleCap = 0;            // rows the sample buffers hold
    // CUDA graphs of the step (jbgpu_world_set_graph): the launches before the pair count
    // readback and those after it, each captured once per buffer arrangement and replayed
    bool graphOn = false;
    std::string graphError;       // set when a capture failed: the world went back to launches
    struct StepGraph {
        uint64_t key[8];
        cudaGraphExec_t exec;
        long long launches;       // kernels in the graph
    };
    std::vector<StepGraph> graphs;
};

namespace {

void graphs_clear(jbgpu_world* w);   // the step graphs bake pointers and arguments: see single_step_graph

int num_sms_of(int dev) {
    int s = 0;
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s > 0 ? s : 1;
}

int alloc_pairs(DevPairs& P, int cap) {
    CK(dalloc(&P.keys, cap)); CK(dalloc(&P.has, cap)); CK(dalloc(&P.n, cap));
    CK(dalloc(&P.b0, cap)); CK(dalloc(&P.b1, cap));
    size_t c4 = (size_t)cap * 4;
    CK(dalloc(&P.pA, c4)); CK(dalloc(&P.pB, c4)); CK(dalloc(&P.wA, c4)); CK(dalloc(&P.wB, c4));
    CK(dalloc(&P.nrm, c4)); CK(dalloc(&P.imp, c4)); CK(dalloc(&P.d1, c4)); CK(dalloc(&P.d2, c4));
    return JBGPU_OK;
}
void free_pairs(DevPairs& P) {
    dfree(P.keys); dfree(P.has); dfree(P.n); dfree(P.b0); dfree(P.b1);
    dfree(P.pA); dfree(P.pB); dfree(P.wA); dfree(P.wB); dfree(P.nrm); dfree(P.imp); dfree(P.d1); dfree(P.d2);
}

// Work buffers whose size follows the pair capacity.
int alloc_pair_work(jbgpu_world* w, int cap) {
    graphs_clear(w);
    DevRows& R = w->rows;
    dfree(R.n_nrm); dfree(R.n_rp1); dfree(R.n_rp2); dfree(R.n_angA); dfree(R.n_angB);
    dfree(R.f_nrm); dfree(R.f_rp1); dfree(R.f_rp2); dfree(R.f_angA); dfree(R.f_angB);
    dfree(R.slot_pair); dfree(R.slot_desc); dfree(R.slot_im); dfree(R.slot_pt0); dfree(R.pt_key);
    size_t c4 = (size_t)cap * 4, c8 = (size_t)cap * 8;
    CK(dalloc(&R.n_nrm, c4)); CK(dalloc(&R.n_rp1, c4)); CK(dalloc(&R.n_rp2, c4)); CK(dalloc(&R.n_angA, c4)); CK(dalloc(&R.n_angB, c4));
    CK(dalloc(&R.f_nrm, c8)); CK(dalloc(&R.f_rp1, c8)); CK(dalloc(&R.f_rp2, c8)); CK(dalloc(&R.f_angA, c8)); CK(dalloc(&R.f_angB, c8));
    CK(dalloc(&R.slot_pair, cap)); CK(dalloc(&R.slot_desc, cap)); CK(dalloc(&R.slot_im, cap));
    CK(dalloc(&R.slot_pt0, cap)); CK(dalloc(&R.pt_key, c4));
    SolverBuffers& S = w->sb;
    dfree(S.flag); dfree(S.candIdx); dfree(S.cand); dfree(S.colourOf); dfree(S.bucket); dfree(S.bucketList);
    dfree(S.md); dfree(S.ml); dfree(S.slotIsl); dfree(S.islList); dfree(S.islChunk); dfree(S.candLocal);
    CK(dalloc(&S.flag, cap)); CK(dalloc(&S.candIdx, cap)); CK(dalloc(&S.cand, cap)); CK(dalloc(&S.colourOf, cap));
    CK(dalloc(&S.bucket, cap)); CK(dalloc(&S.bucketList, cap));
    CK(dalloc(&S.md, cap)); CK(dalloc(&S.ml, cap)); CK(dalloc(&S.slotIsl, cap)); CK(dalloc(&S.islList, cap));
    CK(dalloc(&S.candLocal, cap));
    CK(dalloc(&S.islChunk, (size_t)cap + std::max(w->capBodies, 1)));
    if (S.scanScratch) cudaFree(S.scanScratch);
    CK(cudaMalloc(&S.scanScratch, scan_scratch_bytes(cap)));
    if (w->nb.queue) cudaFree(w->nb.queue);
    CK(cudaMalloc(&w->nb.queue, epa_queue_record_bytes() * (size_t)std::max(cap, 1)));
    dfree(w->nb.ovfQueue); dfree(w->nb.ovfQueue2); dfree(w->nb.pairBucket); dfree(w->nb.perm); dfree(w->nb.blockOff);
    CK(dalloc(&w->nb.ovfQueue, cap)); CK(dalloc(&w->nb.ovfQueue2, cap)); CK(dalloc(&w->nb.pairBucket, cap));
    CK(dalloc(&w->nb.perm, cap));
    {
        int nbk = NB_BUCKETS * ((cap + 255) / 256) + 1;
        CK(dalloc(&w->nb.blockOff, nbk));
        if (w->nb.scanScratch) cudaFree(w->nb.scanScratch);
        CK(cudaMalloc(&w->nb.scanScratch, scan_scratch_bytes(nbk)));
    }
    dfree(w->bb.partners);
    CK(dalloc(&w->bb.partners, cap));
    w->capRows = cap;
    return JBGPU_OK;
}

int grow_bodies(jbgpu_world* w, int need) {
    if (need <= w->capBodies) return JBGPU_OK;
    graphs_clear(w);
    int oldc = w->capBodies;
    int nc = std::max(need, std::max(2 * oldc, w->cfg.initial_body_capacity > 0 ? w->cfg.initial_body_capacity : 1024));
    cudaStream_t s = w->stream;
    DevWorld& d = w->dw;
    size_t keep = (size_t)w->nBodies;
#define G(ptr) CK(dgrow(&d.ptr, oldc, nc, keep, s))
    G(xr0); G(xr1); G(xr2); G(kx0); G(kx1); G(kx2); G(ilv); G(iav); G(hitf); G(linvel); G(angvel); G(iw0); G(iw1); G(iw2); G(iloc); G(force);
    G(torque); G(gravity);
    G(amin); G(amax); G(act); G(deact); G(flags); G(shape); G(group); G(mask); G(world); G(friction); G(restitution);
    G(linSleep); G(angSleep); G(linDamp); G(angDamp); G(island); G(ccdThr); G(ccdRad);
#undef G
    CK(cudaMemsetAsync(d.ccdThr + keep, 0, sizeof(float) * (nc - keep), s));   // CCD off for new bodies
    CK(cudaMemsetAsync(d.ccdRad + keep, 0, sizeof(float) * (nc - keep), s));
    // per-body work buffers (contents not kept)
    BroadphaseBuffers& B = w->bb;
    dfree(B.mkeys); dfree(B.mkeys_alt); dfree(B.sortedBody); dfree(B.vals_alt);
    dfree(B.bvh.left); dfree(B.bvh.right); dfree(B.bvh.lo); dfree(B.bvh.hi); dfree(B.bvh.parent); dfree(B.bvh.leafParent);
    dfree(B.bvh.visit); dfree(B.bvh.node); dfree(B.cnt); dfree(B.off); dfree(B.offPrev); dfree(B.cursor);
    B.offPrevValid = false;
    dfree(B.tcount); dfree(B.tcache);
    CK(dalloc(&B.mkeys, nc)); CK(dalloc(&B.mkeys_alt, nc)); CK(dalloc(&B.sortedBody, nc)); CK(dalloc(&B.vals_alt, nc));
    CK(dalloc(&B.bvh.left, nc)); CK(dalloc(&B.bvh.right, nc)); CK(dalloc(&B.bvh.lo, nc)); CK(dalloc(&B.bvh.hi, nc));
    CK(dalloc(&B.bvh.parent, nc)); CK(dalloc(&B.bvh.leafParent, nc)); CK(dalloc(&B.bvh.visit, nc));
    CK(dalloc(&B.bvh.node, 4 * (size_t)nc)); CK(dalloc(&B.tcount, nc)); CK(dalloc(&B.tcache, (size_t)TRAV_CACHE * nc));
    CK(dalloc(&B.cnt, nc + 1)); CK(dalloc(&B.off, nc + 1)); CK(dalloc(&B.offPrev, nc + 1)); CK(dalloc(&B.cursor, nc + 1));
    if (B.sortScratch) cudaFree(B.sortScratch);
    CK(cudaMalloc(&B.sortScratch, sort_scratch_bytes(nc)));
    if (B.scanScratch) cudaFree(B.scanScratch);
    CK(cudaMalloc(&B.scanScratch, scan_scratch_bytes(nc + 1)));
    SolverBuffers& S = w->sb;
    dfree(S.parent); dfree(S.keepAwake); dfree(S.inactive); dfree(S.claim); dfree(S.taken); dfree(S.posOf);
    dfree(S.islCount); dfree(S.islFill); dfree(S.islStart); dfree(S.segFlag); dfree(S.segIdx);
    dfree(S.islConv); dfree(S.islAcc); dfree(S.islDone);
    CK(dalloc(&S.parent, nc)); CK(dalloc(&S.keepAwake, nc)); CK(dalloc(&S.inactive, nc)); CK(dalloc(&S.claim, nc));
    CK(dalloc(&S.taken, nc)); CK(dalloc(&S.posOf, nc));
    CK(dalloc(&S.islCount, nc + 1)); CK(dalloc(&S.islFill, nc + 1)); CK(dalloc(&S.islStart, nc + 1));
    CK(dalloc(&S.segFlag, nc + 1)); CK(dalloc(&S.segIdx, nc + 1)); CK(dalloc(&S.islConv, nc));
    CK(dalloc(&S.islAcc, 2 * (size_t)nc)); CK(dalloc(&S.islDone, nc));
    if (S.islScratch) cudaFree(S.islScratch);
    CK(cudaMalloc(&S.islScratch, scan_scratch_bytes(nc + 1)));
    if (!S.resTrace) CK(dalloc(&S.resTrace, 2 * (size_t)JBGPU_RESIDUAL_TRACE_MAX));
    w->capBodies = nc;
    return JBGPU_OK;
}

int ensure_pair_capacity(jbgpu_world* w, int buf, int need) {
    if (need <= w->capPairs[buf] && need <= w->capRows) return JBGPU_OK;
    int nc = std::max(need + need / 2 + 64, 2 * w->capPairs[buf]);
    if (need > w->capPairs[buf]) {
        graphs_clear(w);
        free_pairs(w->pairs[buf]);
        int rc = alloc_pairs(w->pairs[buf], nc);
        if (rc) return rc;
        w->capPairs[buf] = nc;
    }
    if (need > w->capRows) {
        int rc = alloc_pair_work(w, std::max(nc, w->capRows));
        if (rc) return rc;
    }
    return JBGPU_OK;
}

// The shape table on the device: the world's shapes by id, then every compound's children
// (a compound's child table entries point at them), and the pools of hull points, tree nodes
// and triangles.  Re-uploaded whole when shapes were added.
int sync_shapes(jbgpu_world* w) {
    if (!w->shapesDirty) return JBGPU_OK;
    const int nu = (int)w->shapes.size(), nc = (int)w->childShapes.size(), ns = nu + nc;
    DevShapes& S = w->dw.sh;
    if (ns > w->capShapes) {
        dfree(S.type); dfree(S.margin); dfree(S.dims); dfree(S.laabb_min); dfree(S.laabb_max); dfree(S.plane);
        dfree(S.hull_off); dfree(S.hull_cnt); dfree(S.child_off); dfree(S.child_cnt); dfree(S.mesh_node_off);
        dfree(S.mesh_node_cnt); dfree(S.mesh_tri_off); dfree(S.mesh_q);
        int c = std::max(ns, 2 * w->capShapes);
        CK(dalloc(&S.type, c)); CK(dalloc(&S.margin, c)); CK(dalloc(&S.dims, c)); CK(dalloc(&S.laabb_min, c));
        CK(dalloc(&S.laabb_max, c)); CK(dalloc(&S.plane, c)); CK(dalloc(&S.hull_off, c)); CK(dalloc(&S.hull_cnt, c));
        CK(dalloc(&S.child_off, c)); CK(dalloc(&S.child_cnt, c)); CK(dalloc(&S.mesh_node_off, c));
        CK(dalloc(&S.mesh_node_cnt, c)); CK(dalloc(&S.mesh_tri_off, c)); CK(dalloc(&S.mesh_q, 3 * (size_t)c));
        w->capShapes = c;
    }
    int nh = (int)w->hullPts.size();
    if (nh > w->capHull || !S.hull_pts) {
        dfree(S.hull_pts);
        int c = std::max(nh, std::max(1, 2 * w->capHull));
        CK(dalloc(&S.hull_pts, c));
        w->capHull = c;
    }
    dfree(S.child_shape); dfree(S.child_xf); dfree(S.mesh_nodes); dfree(S.mesh_tris);
    CK(dalloc(&S.child_shape, nc)); CK(dalloc(&S.child_xf, 3 * (size_t)nc));
    CK(dalloc(&S.mesh_nodes, w->meshNodes.size())); CK(dalloc(&S.mesh_tris, w->meshTris.size()));
    std::vector<int> type(ns), off(ns), cnt(ns), coff(ns), ccnt(ns), noff(ns), ncnt(ns), toff(ns), cshape(nc);
    std::vector<float> margin(ns);
    std::vector<float4> dims(ns), lmin(ns), lmax(ns), plane(ns), q(3 * (size_t)ns);
    for (int i = 0; i < ns; i++) {
        const HostShape& h = i < nu ? w->shapes[i] : w->childShapes[i - nu];
        type[i] = h.type; off[i] = h.hull_off; cnt[i] = h.hull_cnt; margin[i] = h.margin;
        coff[i] = h.child_off; ccnt[i] = h.child_cnt; noff[i] = h.node_off; ncnt[i] = h.node_cnt; toff[i] = h.tri_off;
        dims[i] = make_float4(h.dims[0], h.dims[1], h.dims[2], h.dims[3]);
        lmin[i] = make_float4(h.lmin[0], h.lmin[1], h.lmin[2], 0);
        lmax[i] = make_float4(h.lmax[0], h.lmax[1], h.lmax[2], 0);
        plane[i] = make_float4(h.plane[0], h.plane[1], h.plane[2], h.plane[3]);
        for (int k = 0; k < 3; k++) q[3 * i + k] = make_float4(h.q[4 * k], h.q[4 * k + 1], h.q[4 * k + 2], 0.0f);
    }
    for (int c = 0; c < nc; c++) cshape[c] = nu + c;   // child c is shape nu + c
    cudaStream_t s = w->stream;
    if (ns) {
        CK(cudaMemcpyAsync(S.type, type.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.hull_off, off.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.hull_cnt, cnt.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.margin, margin.data(), sizeof(float) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.dims, dims.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.laabb_min, lmin.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.laabb_max, lmax.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.plane, plane.data(), sizeof(float4) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.child_off, coff.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.child_cnt, ccnt.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.mesh_node_off, noff.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.mesh_node_cnt, ncnt.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.mesh_tri_off, toff.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.mesh_q, q.data(), sizeof(float4) * 3 * ns, cudaMemcpyHostToDevice, s));
    }
    if (nc) {
        CK(cudaMemcpyAsync(S.child_shape, cshape.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(S.child_xf, w->childXf.data(), sizeof(float4) * 3 * nc, cudaMemcpyHostToDevice, s));
    }
    if (!w->meshNodes.empty())
        CK(cudaMemcpyAsync(S.mesh_nodes, w->meshNodes.data(), sizeof(int4) * w->meshNodes.size(), cudaMemcpyHostToDevice, s));
    if (!w->meshTris.empty())
        CK(cudaMemcpyAsync(S.mesh_tris, w->meshTris.data(), sizeof(float4) * w->meshTris.size(), cudaMemcpyHostToDevice, s));
    if (nh) CK(cudaMemcpyAsync(S.hull_pts, w->hullPts.data(), sizeof(float4) * nh, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    w->dw.hasCompound = w->hasCompound ? 1 : 0;
    w->shapesDirty = false;
    return JBGPU_OK;
}

int sync_planes(jbgpu_world* w) {
    if (!w->planesDirty) return JBGPU_OK;
    BroadphaseBuffers& B = w->bb;
    int nw = 1;
    for (int i = 0; i < w->nBodies; i++) nw = std::max(nw, w->hWorld[i] + 1);
    std::vector<std::vector<int>> per(nw);
    int nf = 0, np = 0;
    std::vector<int> finite(nw, 0);
    unsigned kinds = 0;                 // convex shape kinds present
    for (int i = 0; i < w->nBodies; i++) {
        if (w->hFlags[i] & CF_LISTED) { per[w->hWorld[i]].push_back(i); np++; }
        else {
            nf++;
            finite[w->hWorld[i]]++;
            kinds |= 1u << (w->shapes[w->hShape[i]].type & 31);
        }
    }
    // grouping pays with two or more shape kinds, or with GJK pairs (split by contact state),
    // once there are enough pairs to cover its two extra launches
    w->nb.group = (__builtin_popcount(kinds) >= 2 || (kinds & ~(1u << SHAPE_SPHERE)) != 0) && nf >= 4096;
    std::vector<int> list, start(nw + 1, 0);
    for (int k = 0; k < nw; k++) { start[k] = (int)list.size(); list.insert(list.end(), per[k].begin(), per[k].end()); }
    start[nw] = (int)list.size();
    dfree(B.planeList); dfree(B.planeStart); dfree(B.wstart); dfree(B.wend); dfree(B.wroot); dfree(B.bounds); dfree(B.total);
    dfree(B.candBound); dfree(B.segLong);
    CK(dalloc(&B.planeList, std::max<size_t>(1, list.size()))); CK(dalloc(&B.planeStart, nw + 1));
    CK(dalloc(&B.wstart, nw)); CK(dalloc(&B.wend, nw)); CK(dalloc(&B.wroot, nw)); CK(dalloc(&B.bounds, 6)); CK(dalloc(&B.total, 1));
    CK(dalloc(&B.candBound, 1)); CK(dalloc(&B.segLong, 1));
    if (!list.empty()) CK(cudaMemcpy(B.planeList, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.planeStart, start.data(), sizeof(int) * (nw + 1), cudaMemcpyHostToDevice));
    B.nFinite = nf;
    B.nPlanes = np;
    B.nWorlds = nw;
    int bits = 0;
    while ((1 << bits) < nw) bits++;
    B.worldBits = nw > 1 ? bits : 0;
    w->nWorlds = nw;
    w->worldFinite = finite;
    w->bb.built = false;
    w->solverDirty = true;
    w->orderValid = false;
    w->planesDirty = false;
    return JBGPU_OK;
}

DevWorld dev_view(jbgpu_world* w) {
    DevWorld d = w->dw;
    d.nBodies = w->nBodies;
    d.nPairs = w->nPairs;
    return d;
}

int check_status(jbgpu_world* w) {
    int st = 0;
    CK(cudaMemcpyAsync(w->hostPinned, w->dw.ctr + C_STATUS, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    st = *w->hostPinned;
    if (st & ST_TIMEOUT) return fail(JBGPU_ERR_TIMEOUT, "a bounded device wait gave up");
    if (st & ST_EPA_POOL) return fail(JBGPU_ERR_EPA_OVERFLOW, "EPA face pool overflow");
    if (st & ST_CAPACITY) return fail(JBGPU_ERR_CAPACITY, "device capacity exceeded (traversal stack or colours)");
    if (st & ST_BAD_WORLD) return fail(JBGPU_ERR_INVALID_ARGUMENT, "a ray or sweep names a batch world the world does not have");
    if (st & ST_CCD_PLANE)
        return fail(JBGPU_ERR_UNSUPPORTED, "a CCD sweep reached a static plane, where the reference throws "
                                           "(CollisionWorld.objectQuerySingle's concave branch)");
    return JBGPU_OK;
}

// ---- stages --------------------------------------------------------------------------------
int stage_pairs_fill(jbgpu_world* w, int total);
int stage_pairs(jbgpu_world* w) {
    DevWorld d = dev_view(w);
    cudaStream_t s = w->stream;
    w->prof.mark(PH_PAIR_COUNT, 0, s);
    broadphase_run_count(d, w->bb, s);
    w->orderValid = true;
    w->prof.mark(PH_PAIR_COUNT, 1, s);
    CK(cudaMemcpyAsync(w->hostPinned, w->bb.total, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(w->hostPinned + 2, w->bb.candBound, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    w->candBound = w->hostPinned[2];
    return stage_pairs_fill(w, *w->hostPinned);
}

// The pair stage after the count: buffers for `total` pairs, fill, persistence.
int stage_pairs_fill(jbgpu_world* w, int total) {
    DevWorld d = dev_view(w);
    cudaStream_t s = w->stream;
    int nxt = w->cur ^ 1;
    int rc = ensure_pair_capacity(w, nxt, total);
    if (rc) return rc;
    if (w->hasMesh && concave_reserve(w->nb, w->capRows, w->candBound, s) < 0)
        return fail(JBGPU_ERR_CUDA, "concave pass buffers");
    w->prof.mark(PH_PAIR_FILL, 0, s);
    broadphase_run_fill(d, w->bb, w->pairs[nxt], w->capRows, s);
    broadphase_persist(d, w->bb, w->pairs[nxt], w->pairs[w->cur], total, w->nPairs, s);
    w->prof.mark(PH_PAIR_FILL, 1, s);
    w->cur = nxt;
    w->nPairs = total;
    CK(cudaMemcpyAsync(w->dw.ctr + C_PAIRS, w->bb.total, sizeof(int), cudaMemcpyDeviceToDevice, s));
    return JBGPU_OK;
}

// Solver parts and the body order they index: the broadphase leaf order when it covers every
// body, else finite bodies grouped by world in index order, built here.
int prepare_solver(jbgpu_world* w) {
    SolverBuffers& S = w->sb;
    const int nf = w->bb.nFinite;
    if (w->solverDirty) {
        graphs_clear(w);
        int rc = solver_configure(S, nf, w->worldFinite, w->sms, w->cfg.solver_parts,
                                  w->cfg.solver_threads ? w->cfg.solver_threads : SOLVER_THREADS, w->cfg.solver_smem_bodies);
        if (rc) return fail(rc, "solver part tables");
        w->solverDirty = false;
    }
    if (w->orderValid) {
        S.order = w->bb.sortedBody;
        return JBGPU_OK;
    }
    std::vector<int> at(w->nWorlds + 1, 0), ord(std::max(nf, 1));
    for (int q = 0; q < w->nWorlds; q++) at[q + 1] = at[q] + w->worldFinite[q];
    for (int i = 0; i < w->nBodies; i++)
        if (!(w->hFlags[i] & CF_LISTED)) ord[at[w->hWorld[i]]++] = i;
    dfree(S.orderFallback);
    CK(dalloc(&S.orderFallback, ord.size()));
    CK(cudaMemcpyAsync(S.orderFallback, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    S.order = S.orderFallback;
    return JBGPU_OK;
}

int run_stage(jbgpu_world* w, int stage, float dt) {
    cudaStream_t s = w->stream;
    DevWorld d = dev_view(w);
    const Prof& P = w->prof;
    switch (stage) {
    case JBGPU_STAGE_APPLY_GRAVITY: P.mark(PH_OTHER, 0, s); launch_apply_gravity(d, s); P.mark(PH_OTHER, 1, s); break;
    case JBGPU_STAGE_PREDICT: P.mark(PH_PREDICT, 0, s); launch_predict(d, dt, s); P.mark(PH_PREDICT, 1, s); break;
    case JBGPU_STAGE_AABB: P.mark(PH_AABB, 0, s); launch_aabb(d, s); P.mark(PH_AABB, 1, s); break;
    case JBGPU_STAGE_PAIRS: { int rc = stage_pairs(w); if (rc) return rc; break; }
    case JBGPU_STAGE_NARROWPHASE:
        CK(cudaMemsetAsync(w->dw.ctr + C_GJK, 0, sizeof(int) * 2, s));
        narrowphase_launch(d, w->pairs[w->cur], w->nPairs, w->nb, s, &P);
        if (w->hasMesh) {
            P.mark(PH_CONCAVE, 0, s);
            if (concave_launch(d, w->pairs[w->cur], w->nPairs, nullptr, w->nb, w->hostPinned + 8, s))
                return fail(JBGPU_ERR_CUDA, "concave narrowphase pass failed");
            P.mark(PH_CONCAVE, 1, s);
        }
        break;
    case JBGPU_STAGE_ISLANDS:
        P.mark(PH_ISLANDS, 0, s);
        CK(cudaMemsetAsync(w->dw.ctr + C_ISLANDS, 0, sizeof(int) * 4, s));
        islands_launch(d, w->pairs[w->cur], w->nPairs, w->sb, s);
        P.mark(PH_ISLANDS, 1, s);
        break;
    case JBGPU_STAGE_SOLVE: {
        int rc = prepare_solver(w);
        if (rc) return rc;
        CK(cudaMemsetAsync(w->dw.ctr + C_ROWS, 0, sizeof(int), s));
        SolverLearn learn;
        MlpDev md;
        if (w->mlp) {
            md = mlp_view(w->mlp);
            learn.mlp = &md;
        }
        if (w->logSamples) {
            if (w->sampleCap < w->capRows) {
                dfree(w->sampleX);
                dfree(w->sampleT);
                w->sampleCap = 0;
                CK(dalloc(&w->sampleX, (size_t)w->capRows * 4 * JBGPU_MLP_INPUTS));
                CK(dalloc(&w->sampleT, (size_t)w->capRows * 4 * JBGPU_MLP_OUTPUTS));
                w->sampleCap = w->capRows;
            }
            learn.sampleX = w->sampleX;
            learn.sampleT = w->sampleT;
            learn.allPoints = w->logAll ? 1 : 0;
        }
        solve_launch_learn(d, w->pairs[w->cur], w->nPairs, w->rows, w->sb, dt, s, &P, learn);
        break;
    }
    case JBGPU_STAGE_INTEGRATE:
        P.mark(PH_INTEGRATE, 0, s);
        if (w->ccdOn) {
            int rc = ccd_integrate(d, w->pairs[w->cur], w->nPairs, w->pairCountDev, w->cb, dt, w->sms, s);
            if (rc) return fail(rc, "CCD integration failed");
        } else {
            launch_integrate(d, dt, s);
        }
        P.mark(PH_INTEGRATE, 1, s);
        break;
    case JBGPU_STAGE_ACTIVATION: P.mark(PH_ACTIVATION, 0, s); launch_activation(d, dt, s); P.mark(PH_ACTIVATION, 1, s); break;
    case JBGPU_STAGE_CLEAR_FORCES: launch_clear_forces(d, s); break;
    case JBGPU_STAGE_SAVE_KINEMATIC: launch_save_kinematic(d, dt, s); break;
    default: return fail(JBGPU_ERR_INVALID_ARGUMENT, "unknown stage");
    }
    CK(cudaGetLastError());
    return JBGPU_OK;
}

// Joints to the device: arrays grown to the joint count, the colouring (first fit in index
// order: a joint takes the lowest colour no earlier joint on one of its dynamic bodies holds;
// static and kinematic bodies take no impulse, so they do not order joints) and the solve order
// by (colour, index).
int sync_joints(jbgpu_world* w) {
    if (!w->jointsDirty) return JBGPU_OK;
    DevJoints& J = w->sb.J;
    const int n = (int)w->jA.size();
    if (n > w->capJoints) {
        dfree(J.a); dfree(J.b); dfree(J.pivA); dfree(J.pivB); dfree(J.set); dfree(J.order); dfree(J.colStart);
        dfree(J.r1); dfree(J.r2); dfree(J.dep); dfree(J.imp); dfree(J.act);
        dfree(J.kind); dfree(J.set2); dfree(J.frame); dfree(J.hs); dfree(J.d6set);
        const int c = std::max(n, 2 * w->capJoints);
        CK(dalloc(&J.a, c)); CK(dalloc(&J.b, c)); CK(dalloc(&J.pivA, c)); CK(dalloc(&J.pivB, c)); CK(dalloc(&J.set, c));
        CK(dalloc(&J.kind, c)); CK(dalloc(&J.set2, c)); CK(dalloc(&J.frame, 6 * c)); CK(dalloc(&J.hs, JOINT_STEP_F4 * c));
        CK(dalloc(&J.d6set, D6_SET_F4 * (size_t)c));
        CK(dalloc(&J.order, c)); CK(dalloc(&J.colStart, c + 1)); CK(dalloc(&J.r1, c)); CK(dalloc(&J.r2, c));
        CK(dalloc(&J.dep, c)); CK(dalloc(&J.imp, c)); CK(dalloc(&J.act, c));
        CK(cudaMemset(J.imp, 0, sizeof(float) * c));
        w->capJoints = c;
    }
    auto dynBody = [&](int b) { return b >= 0 && !(w->hFlags[b] & (CF_STATIC | CF_KINEMATIC)); };
    std::vector<std::vector<int>> used(w->nBodies);
    std::vector<std::pair<int, int>> ck(n);
    int nCol = 0;
    for (int k = 0; k < n; k++) {
        int c = 0;
        for (;; c++) {
            bool clash = false;
            for (int b : {w->jA[k], w->jB[k]})
                if (dynBody(b))
                    for (int u : used[b]) clash = clash || u == c;
            if (!clash) break;
        }
        for (int b : {w->jA[k], w->jB[k]})
            if (dynBody(b)) used[b].push_back(c);
        ck[k] = {c, k};
        nCol = std::max(nCol, c + 1);
    }
    std::sort(ck.begin(), ck.end());
    std::vector<int> order(n), colStart(nCol + 1, 0);
    for (int k = 0; k < n; k++) { order[k] = ck[k].second; colStart[ck[k].first + 1]++; }
    for (int c = 0; c < nCol; c++) colStart[c + 1] += colStart[c];
    cudaStream_t s = w->stream;
    CK(cudaMemcpyAsync(J.a, w->jA.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.b, w->jB.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.pivA, w->jPivA.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.pivB, w->jPivB.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.set, w->jSet.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.kind, w->jKind.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.set2, w->jSet2.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.frame, w->jFrame.data(), sizeof(float4) * 6 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.d6set, w->jD6.data(), sizeof(float4) * D6_SET_F4 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.order, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(J.colStart, colStart.data(), sizeof(int) * (nCol + 1), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    J.n = n;
    J.nCol = nCol;
    w->jointsDirty = false;
    return JBGPU_OK;
}

int prepare(jbgpu_world* w) {
    CK(cudaSetDevice(w->device));
    if (w->shapesDirty || w->planesDirty || w->jointsDirty || w->solverDirty) graphs_clear(w);
    int rc = sync_shapes(w);
    if (rc) return rc;
    if (!w->aabbRefresh.empty()) {   // refitted meshes: updateSingleAabb of their bodies
        if (w->nBodies > 0) {
            DevWorld d = dev_view(w);
            for (int s : w->aabbRefresh) { k_shape_aabbs<<<(w->nBodies + 255) / 256, 256, 0, w->stream>>>(d, s); note_launch(); }
            CK(cudaGetLastError());
        }
        w->aabbRefresh.clear();
    }
    rc = sync_planes(w);
    if (rc) return rc;
    return sync_joints(w);
}

void graphs_clear(jbgpu_world* w) {
    for (auto& g : w->graphs) cudaGraphExecDestroy(g.exec);
    w->graphs.clear();
}

// Narrowphase and islands of one step: the island unions run on the second stream while the
// narrowphase runs on the world's stream; sleep decisions and manifold selection follow both.
// cntp (nullable): the pair count on the device, w->nPairs then being an upper bound.
int narrow_and_islands(jbgpu_world* w, const int* cntp = nullptr) {
    cudaStream_t s = w->stream, a = w->aux;
    DevWorld d = dev_view(w);
    CK(cudaEventRecord(w->evFork, s));
    CK(cudaStreamWaitEvent(a, w->evFork, 0));
    CK(cudaMemsetAsync(w->dw.ctr + C_ISLANDS, 0, sizeof(int) * 4, a));
    islands_launch_unions(d, w->pairs[w->cur], w->nPairs, w->sb, a, cntp);
    CK(cudaEventRecord(w->evJoin, a));
    CK(cudaMemsetAsync(w->dw.ctr + C_GJK, 0, sizeof(int) * 2, s));
    narrowphase_launch(d, w->pairs[w->cur], w->nPairs, w->nb, s, &w->prof, cntp);
    if (w->hasMesh) {   // buffers reserved for the count pass's bound (stage_pairs_fill, single_step_graph)
        w->prof.mark(PH_CONCAVE, 0, s);
        if (concave_launch_bounded(d, w->pairs[w->cur], w->nPairs, cntp, w->nb, w->candBound, s))
            return fail(JBGPU_ERR_CUDA, "concave narrowphase pass failed");
        w->prof.mark(PH_CONCAVE, 1, s);
    }
    CK(cudaStreamWaitEvent(s, w->evJoin, 0));
    w->prof.mark(PH_ISLANDS, 0, s);
    islands_launch_select(d, w->pairs[w->cur], w->nPairs, w->sb, s, cntp);
    w->prof.mark(PH_ISLANDS, 1, s);
    CK(cudaGetLastError());
    return JBGPU_OK;
}

// ---- the step as two CUDA graphs ------------------------------------------------------------
// Graph A holds the launches up to the pair count (predict, aabbs, the broadphase count with the
// tree rebuild or refit) and copies the count to pinned host memory; the host reads it (the one
// synchronisation of a step, as in the launch path), grows the pair buffers if needed, and
// replays graph B: pair fill and persistence, narrowphase with the islands on the second stream,
// the solver, integration and activation.  B's kernels read the pair count from the device
// (w.ctr[C_PAIRS], the broadphase total) and are sized by the pair capacity.  Launches bake
// their pointers and host-side arguments, so each graph is kept per arrangement of the
// alternating buffers (pair arrays, per-owner offsets), the tree path (rebuild or refit) and dt;
// anything else that changes a buffer or an argument clears them all (graphs_clear).  The host
// state the launch functions change while a graph is captured (tree age, offset swap) is
// changed by hand when the graph is replayed.
namespace {
constexpr int GRAPH_FALLBACK = -1000;   // a capture failed: the step goes on with launches

template <class F>
int capture_or_replay(jbgpu_world* w, const uint64_t key[8], F&& body, bool& captured) {
    captured = false;
    for (auto& g : w->graphs)
        if (std::equal(g.key, g.key + 8, key)) {
            CK(cudaGraphLaunch(g.exec, w->stream));
            g_launches.fetch_add(g.launches, std::memory_order_relaxed);
            return JBGPU_OK;
        }
    cudaStream_t s = w->stream;
    const long long l0 = g_launches.load();
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        w->graphError = "stream capture could not begin";
        cudaGetLastError();
        return GRAPH_FALLBACK;
    }
    int rc = body();
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    const long long n = g_launches.load() - l0;
    g_launches.fetch_sub(n, std::memory_order_relaxed);
    cudaGraphExec_t exec = nullptr;
    if (rc == JBGPU_OK && e == cudaSuccess && graph) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (rc != JBGPU_OK || e != cudaSuccess || !exec) {
        w->graphError = std::string("graph capture failed: ") + (rc != JBGPU_OK ? g_err : cudaGetErrorString(e));
        cudaGetLastError();
        return GRAPH_FALLBACK;
    }
    jbgpu_world::StepGraph g;
    std::copy(key, key + 8, g.key);
    g.exec = exec;
    g.launches = n;
    w->graphs.push_back(g);
    captured = true;
    CK(cudaGraphLaunch(exec, s));
    g_launches.fetch_add(n, std::memory_order_relaxed);
    return JBGPU_OK;
}

uint64_t fbits64(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

int single_step_graph(jbgpu_world* w, float dt) {
    cudaStream_t s = w->stream;
    BroadphaseBuffers& B = w->bb;
    const bool rebuild = !(B.built && B.sinceBuild + 1 < B.rebuildInterval);
    const bool builtBefore = B.built;
    const int ageBefore = B.sinceBuild;
    const uint64_t ka[8] = {1, (uint64_t)rebuild, (uint64_t)(uintptr_t)B.off, (uint64_t)(uintptr_t)B.offPrev,
                            fbits64(dt), 0, 0, 0};
    bool captured = false;
    int rc = capture_or_replay(w, ka, [&]() -> int {
        DevWorld d = dev_view(w);
        launch_predict(d, dt, s);
        launch_aabb(d, s);
        broadphase_run_count(d, B, s);
        CK(cudaMemcpyAsync(w->hostPinned + 1, B.total, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(w->hostPinned + 2, B.candBound, sizeof(int), cudaMemcpyDeviceToHost, s));
        return JBGPU_OK;
    }, captured);
    if (rc == GRAPH_FALLBACK) {            // nothing ran: undo the capture's host side
        B.built = builtBefore;
        B.sinceBuild = ageBefore;
        return GRAPH_FALLBACK;
    }
    if (rc) return rc;
    if (!captured) {                       // what broadphase_run_count does on the host
        if (rebuild) { B.built = true; B.sinceBuild = 0; }
        else B.sinceBuild++;
    }
    w->orderValid = true;
    CK(cudaStreamSynchronize(s));
    const int total = w->hostPinned[1];
    w->candBound = w->hostPinned[2];
    const int nxt = w->cur ^ 1;
    const int capBefore = w->capRows;
    void* keysBefore = w->pairs[nxt].keys;
    if ((rc = ensure_pair_capacity(w, nxt, total))) return rc;
    if (w->capRows != capBefore || w->pairs[nxt].keys != keysBefore) graphs_clear(w);
    if (w->hasMesh) {   // the concave pass's buffers for this step's bound, before graph B is replayed
        const int moved = concave_reserve(w->nb, w->capRows, w->candBound, s);
        if (moved < 0) return fail(JBGPU_ERR_CUDA, "concave pass buffers");
        if (moved) graphs_clear(w);
    }
    if ((rc = prepare_solver(w))) return rc;
    const int old = w->cur;
    int* const offBefore = B.off;
    int* const offPrevBefore = B.offPrev;
    const bool offValidBefore = B.offPrevValid;
    const int nPairsBefore = w->nPairs;
    const uint64_t kb[8] = {2, (uint64_t)(uintptr_t)w->pairs[old].keys, (uint64_t)(uintptr_t)w->pairs[nxt].keys,
                            (uint64_t)(uintptr_t)B.off, (uint64_t)(uintptr_t)B.offPrev, (uint64_t)B.offPrevValid,
                            (uint64_t)w->capRows, fbits64(dt)};
    const int bound = w->capRows;
    int* cnt = w->dw.ctr + C_PAIRS;
    w->cur = nxt;
    w->nPairs = bound;                     // launches are sized by the capacity ...
    rc = capture_or_replay(w, kb, [&]() -> int {
        DevWorld d = dev_view(w);
        w->pairCountDev = cnt;
        struct Reset { jbgpu_world* w; ~Reset() { w->pairCountDev = nullptr; } } reset{w};
        broadphase_run_fill(d, B, w->pairs[nxt], bound, s);
        broadphase_persist(d, B, w->pairs[nxt], w->pairs[old], bound, w->capPairs[old], s, B.total, cnt);
        CK(cudaMemcpyAsync(cnt, B.total, sizeof(int), cudaMemcpyDeviceToDevice, s));
        int r = narrow_and_islands(w, cnt);   // ... and read the count from the device
        if (r) return r;
        static const int rest[] = {JBGPU_STAGE_SOLVE, JBGPU_STAGE_INTEGRATE, JBGPU_STAGE_ACTIVATION};
        for (int st : rest)
            if ((r = run_stage(w, st, dt))) return r;
        return JBGPU_OK;
    }, captured);
    if (rc == GRAPH_FALLBACK) {            // the count ran; the rest with launches
        B.off = offBefore;
        B.offPrev = offPrevBefore;
        B.offPrevValid = offValidBefore;
        w->cur = old;
        w->nPairs = nPairsBefore;
        static const int rest[] = {JBGPU_STAGE_NARROWPHASE, JBGPU_STAGE_SOLVE, JBGPU_STAGE_INTEGRATE,
                                   JBGPU_STAGE_ACTIVATION};
        if ((rc = stage_pairs_fill(w, total))) return rc;
        for (int st : rest)
            if ((rc = st == JBGPU_STAGE_NARROWPHASE ? narrow_and_islands(w) : run_stage(w, st, dt))) return rc;
        w->steps++;
        return JBGPU_OK;
    }
    w->nPairs = total;
    if (rc) return rc;
    if (!captured) {                       // broadphase_persist's host side
        std::swap(B.off, B.offPrev);
        B.offPrevValid = true;
    }
    w->steps++;
    return JBGPU_OK;
}

bool graph_usable(const jbgpu_world* w) {
    return w->graphOn && w->graphError.empty() && !w->prof.active() && !w->mlp && !w->logSamples && w->nBodies > 0;
}
}  // namespace

int single_step(jbgpu_world* w, float dt) {
    if (w->ccdOn && ccd_reserve(w->cb, w->nBodies, w->sms)) return fail(JBGPU_ERR_CUDA, "CCD buffers");
    if (graph_usable(w)) {
        int rc = single_step_graph(w, dt);
        if (rc != GRAPH_FALLBACK) return rc;   // else the capture failed before anything ran
    }
    static const int order[] = {JBGPU_STAGE_PREDICT, JBGPU_STAGE_AABB, JBGPU_STAGE_PAIRS, JBGPU_STAGE_NARROWPHASE,
                                JBGPU_STAGE_SOLVE, JBGPU_STAGE_INTEGRATE, JBGPU_STAGE_ACTIVATION};
    for (int st : order) {
        int rc = st == JBGPU_STAGE_NARROWPHASE ? narrow_and_islands(w) : run_stage(w, st, dt);
        if (rc) return rc;
    }
    w->steps++;
    if (w->prof.active()) {
        int* h = w->profHist + (size_t)w->prof.step * (C_NCTR + 1);
        CK(cudaMemcpyAsync(h, w->dw.ctr, sizeof(int) * C_NCTR, cudaMemcpyDeviceToDevice, w->stream));
        CK(cudaMemcpyAsync(h + C_NCTR, w->sb.nCand, sizeof(int), cudaMemcpyDeviceToDevice, w->stream));
        w->prof.step++;
    }
    return JBGPU_OK;
}

void free_prof(Prof& p) {
    if (p.ev) {
        for (size_t i = 0; i < (size_t)p.maxSteps * NUM_PHASES * 2; i++) cudaEventDestroy(p.ev[i]);
        delete[] p.ev;
    }
    p.ev = nullptr;
    p.maxSteps = 0;
    p.step = 0;
}

// RigidBody setup arithmetic on the host (dynamics/RigidBody.java:121-164,207-217,301-312):
// binary32 operations, no contraction (this file's host code is built with -ffp-contract=off).
struct BodyInit {
    float invMass, il[3], grav[3], linDamp, angDamp;
    int flags, group, mask;
};

}  // namespace

// Kernel: invInertiaTensorWorld and the creation-time proxy aabb (shape aabb without the
// contact threshold, CollisionWorld.addCollisionObject) for a range of new bodies.
__global__ void k_init_bodies(DevWorld w, int first, int count);
__global__ void k_add_forces(DevWorld w, const float* f, const float* t);
__global__ void k_pack_transforms(DevWorld w, float* out);
__global__ void k_pack_interpolated(DevWorld w, float t, float* out);

namespace {
int ensure_io(jbgpu_world* w) {
    if (w->capIo >= w->nBodies && w->ioStage) return JBGPU_OK;
    if (w->ioStage) cudaFree(w->ioStage);
    w->ioStage = nullptr;
    int c = std::max(w->nBodies, w->capBodies);
    CK(cudaMalloc(&w->ioStage, sizeof(float) * 12 * (size_t)std::max(c, 1)));
    w->capIo = c;
    return JBGPU_OK;
}
}  // namespace

namespace bodyprops {
// Per-body values written at the listed bodies (the listed bodies are distinct).
__global__ void k_scatter(float* dst, const int* idx, const float* v, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[idx[k]] = v[k];
}

// n body indices, each in range and listed once.
int check_distinct(const jbgpu_world* w, const int32_t* bodies, int n) {
    std::vector<char> seen(w->nBodies, 0);
    for (int k = 0; k < n; k++) {
        if (bodies[k] < 0 || bodies[k] >= w->nBodies) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad body index");
        if (seen[bodies[k]]) return fail(JBGPU_ERR_INVALID_ARGUMENT, "a body listed twice in one call");
        seen[bodies[k]] = 1;
    }
    return JBGPU_OK;
}

// The tick callback after a substep: the substep's status is checked first (a later call from
// the callback resets the status word), the world is brought up to date after it (the callback
// may have added or removed bodies or joints).
int after_substep(jbgpu_world* w, float dt) {
    if (!w->tickCb) return JBGPU_OK;
    int rc = check_status(w);
    if (rc) return rc;
    w->inTick = true;
    w->tickCb(w, dt, w->tickUser);
    w->inTick = false;
    if ((rc = prepare(w))) return rc;
    CK(cudaMemsetAsync(w->dw.ctr + C_STATUS, 0, sizeof(int), w->stream));
    return JBGPU_OK;
}
}  // namespace bodyprops

namespace removal {
// Body removal: dst[j] = src[from[j]] for every kept body, and the pairs whose bodies both stay,
// moved to the other pair buffer in their order with the bodies renumbered.
template <class T>
__global__ void k_gather(const T* src, T* dst, const int* from, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) dst[j] = src[from[j]];
}
__global__ void k_pairs_keep(DevPairs P, int nPairs, const int* newIndex, int* flag) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPairs) return;
    const uint64_t k = P.keys[p];
    flag[p] = newIndex[key_owner(k)] >= 0 && newIndex[key_partner(k)] >= 0;
}
__global__ void k_pairs_move(DevPairs S, DevPairs D, int nPairs, const int* flag, const int* pos, const int* newIndex) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPairs || !flag[p]) return;
    const int q = pos[p];
    const uint64_t k = S.keys[p];
    D.keys[q] = ((uint64_t)(unsigned)newIndex[key_owner(k)] << 32) | ((uint64_t)key_sub(k) << 24) |
                (uint64_t)(unsigned)newIndex[key_partner(k)];
    D.has[q] = S.has[p];
    D.n[q] = S.n[p];
    D.b0[q] = S.b0[p] >= 0 ? newIndex[S.b0[p]] : S.b0[p];
    D.b1[q] = S.b1[p] >= 0 ? newIndex[S.b1[p]] : S.b1[p];
    for (int j = 0; j < 4; j++) {
        const int s = 4 * p + j, d = 4 * q + j;
        D.pA[d] = S.pA[s]; D.pB[d] = S.pB[s]; D.wA[d] = S.wA[s]; D.wB[d] = S.wB[s];
        D.nrm[d] = S.nrm[s]; D.imp[d] = S.imp[s]; D.d1[d] = S.d1[s]; D.d2[d] = S.d2[s];
    }
}
template <class T>
int gather_array(T* a, const int* from, int n, void* tmp, cudaStream_t s) {
    if (n == 0) return JBGPU_OK;
    k_gather<T><<<(n + 255) / 256, 256, 0, s>>>(a, (T*)tmp, from, n);
    note_launch();
    CK(cudaMemcpyAsync(a, tmp, sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
    return JBGPU_OK;
}
}  // namespace removal

extern "C" {

const char* jbgpu_version(void) { return "jbgpu 0.1 (sm_103a)"; }
int64_t jbgpu_launch_count(void) { return g_launches.load(); }
const char* jbgpu_last_error(void) { return g_err.c_str(); }

void jbgpu_config_default(jbgpu_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->gravity[0] = 0.0f; c->gravity[1] = -10.0f; c->gravity[2] = 0.0f;
    c->contact_breaking_threshold = 0.02f;
    c->deactivation_time = 2.0f;
    c->disable_deactivation = 0;
    c->num_iterations = 10;
    c->erp = 0.2f;
    c->warmstarting_factor = 0.85f;
    c->linear_slop = 0.0f;
    c->solver_mode = JBGPU_SOLVER_CACHE_FRIENDLY | JBGPU_SOLVER_USE_WARMSTARTING;
    c->device = 0;
    c->initial_body_capacity = 1024;
    c->pairs_per_body = 16;
    c->broadphase_rebuild_interval = 4;
    c->step_graphs = 1;
}

namespace {
// java.lang.Math.min / max on floats
float jmin_h(float a, float b) {
    if (a != a) return a;
    if (a == 0.0f && b == 0.0f) return std::signbit(b) ? b : a;
    return a <= b ? a : b;
}
float jmax_h(float a, float b) {
    if (a != a) return a;
    if (a == 0.0f && b == 0.0f) return std::signbit(a) ? b : a;
    return a >= b ? a : b;
}
float dot3_h(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// A convex shape record from its descriptor (BoxShape, SphereShape, CapsuleShape,
// ConvexHullShape constructors; hull points appended to pts).
int convex_record(std::vector<float4>& pts, const jbgpu_shape_desc& d, HostShape& h) {
    std::memset(&h, 0, sizeof(h));
    h.type = d.type;
    h.margin = 0.04f;
    switch (d.type) {
    case JBGPU_SHAPE_BOX:       // BoxShape: implicit dims = halfExtents * scaling - margin
        for (int k = 0; k < 3; k++) { volatile float v = d.params[k] * 1.0f; h.dims[k] = v - 0.04f; }
        return JBGPU_OK;
    case JBGPU_SHAPE_SPHERE:    // SphereShape: radius in dims.x, margin == radius
        h.dims[0] = d.params[0];
        h.margin = d.params[0];
        return JBGPU_OK;
    case JBGPU_SHAPE_CAPSULE:   // CapsuleShape(radius, height), up axis y
        h.dims[0] = d.params[0]; h.dims[1] = 0.5f * d.params[1]; h.dims[2] = d.params[0]; h.dims[3] = 1.0f;
        return JBGPU_OK;
    case JBGPU_SHAPE_CONVEX_HULL: {
        if (!d.points || d.num_points <= 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "hull without points");
        h.hull_off = (int)pts.size();
        h.hull_cnt = d.num_points;
        for (int k = 0; k < d.num_points; k++)
            pts.push_back(make_float4(d.points[3 * k], d.points[3 * k + 1], d.points[3 * k + 2], 0.0f));
        for (int a = 0; a < 3; a++) {   // PolyhedralConvexShape.recalcLocalAabb: strict > argmax
            float bp = -1e30f, bm = -1e30f, vp = 0.0f, vm = 0.0f;
            for (int k = 0; k < d.num_points; k++) {
                float x = d.points[3 * k + a];
                if (x > bp) { bp = x; vp = x; }
                if (-x > bm) { bm = -x; vm = x; }
            }
            h.lmax[a] = vp + 0.04f;
            h.lmin[a] = vm - 0.04f;
        }
        return JBGPU_OK;
    }
    }
    return fail(JBGPU_ERR_UNSUPPORTED, "a compound child must be a box, sphere, capsule or convex hull");
}

// getAabb of a convex record at a transform t (12 floats: basis rows, origin), the device's
// shape_aabb on the host: BoxShape via AabbUtil2.transformAabb, SphereShape, CapsuleShape,
// PolyhedralConvexShape.
void convex_record_aabb(const HostShape& h, const float* t, float mn[3], float mx[3]) {
    float ab[9], c[3], he[3];
    for (int i = 0; i < 9; i++) ab[i] = std::fabs(t[i]);
    const float m = h.margin;
    for (int k = 0; k < 3; k++) c[k] = t[9 + k];
    if (h.type == JBGPU_SHAPE_SPHERE) {
        for (int k = 0; k < 3; k++) { mn[k] = c[k] - m; mx[k] = c[k] + m; }
        return;
    }
    if (h.type == JBGPU_SHAPE_BOX) {
        for (int k = 0; k < 3; k++) he[k] = h.dims[k] + m;
    } else if (h.type == JBGPU_SHAPE_CAPSULE) {
        const float r = h.dims[0];
        he[0] = r; he[1] = r + h.dims[1]; he[2] = r;
        for (int k = 0; k < 3; k++) he[k] = he[k] + m;
    } else {   // hull: transformAabb(localMin, localMax, margin, t)
        float lc[3];
        for (int k = 0; k < 3; k++) {
            he[k] = (h.lmax[k] - h.lmin[k]) * 0.5f;
            he[k] = he[k] + m;
            lc[k] = (h.lmax[k] + h.lmin[k]) * 0.5f;
        }
        for (int k = 0; k < 3; k++) c[k] = dot3_h(lc, t + 3 * k) + t[9 + k];
    }
    for (int k = 0; k < 3; k++) {
        const float e = dot3_h(ab + 3 * k, he);
        mn[k] = c[k] - e;
        mx[k] = c[k] + e;
    }
}

// CompoundShape local aabb: the union of its children's aabbs at their transforms
// (CompoundShape.addChildShape, CompoundShape.java:59-91).
void compound_local_aabb(const std::vector<HostShape>& ch, const float* xf, int n, float lmin[3], float lmax[3]) {
    for (int k = 0; k < 3; k++) { lmin[k] = 1e30f; lmax[k] = -1e30f; }
    for (int i = 0; i < n; i++) {
        float mn[3], mx[3];
        convex_record_aabb(ch[i], xf + 12 * i, mn, mx);
        for (int k = 0; k < 3; k++) { lmin[k] = jmin_h(lmin[k], mn[k]); lmax[k] = jmax_h(lmax[k], mx[k]); }
    }
}
// The vertices of a TRIANGLE_MESH descriptor as the reference reads them: each multiplied by the
// mesh interface's scaling (VertexData.getTriangle, VertexData.java:50-55), which
// BvhTriangleMeshShape.setLocalScaling sets - and rebuilds the tree over - only when it differs
// from the current (1, 1, 1) by a squared length above SIMD_EPSILON
// (BvhTriangleMeshShape.java:195-212).  params[1..3] all zero: no scaling.
const float* scaled_vertices(const float* points, int n, const float s[3], std::vector<float>& buf) {
    const float sx = s[0], sy = s[1], sz = s[2];
    if (!points || n <= 0 || (sx == 0.0f && sy == 0.0f && sz == 0.0f)) return points;
    const float dx = 1.0f - sx, dy = 1.0f - sy, dz = 1.0f - sz;
    const float l2 = dx * dx + dy * dy + dz * dz;
    if (!(l2 > 1.1920929e-7f)) return points;
    buf.resize((size_t)3 * n);
    for (int i = 0; i < n; i++) {
        buf[3 * i] = points[3 * i] * sx;
        buf[3 * i + 1] = points[3 * i + 1] * sy;
        buf[3 * i + 2] = points[3 * i + 2] * sz;
    }
    return buf.data();
}
const float* mesh_vertices(const jbgpu_shape_desc& d, std::vector<float>& buf) {
    return scaled_vertices(d.points, d.num_points, d.params + 1, buf);
}
}  // namespace

int jbgpu_shape_mesh_bvh(const jbgpu_shape_desc* d, int32_t* nodes, int32_t capacity, int32_t* n, float aabb[6]) {
    if (!d || !n || d->type != JBGPU_SHAPE_TRIANGLE_MESH || capacity < 0 || (capacity > 0 && !nodes))
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "a TRIANGLE_MESH descriptor, a count pointer and a node buffer");
    MeshBvh m;
    std::vector<float> scaled;
    if (build_mesh_bvh(mesh_vertices(*d, scaled), d->num_points, d->indices, d->num_triangles, m))
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "a triangle mesh needs vertices, 1 .. 2^21-1 triangles and indices "
                                                "within the vertex array");
    *n = (int)m.nodes.size();
    if (aabb)
        for (int k = 0; k < 3; k++) { aabb[k] = m.lmin[k]; aabb[3 + k] = m.lmax[k]; }
    if (*n > capacity) return fail(JBGPU_ERR_CAPACITY, "node buffer too small");
    for (int i = 0; i < *n; i++) {
        nodes[4 * i] = m.nodes[i].x; nodes[4 * i + 1] = m.nodes[i].y;
        nodes[4 * i + 2] = m.nodes[i].z; nodes[4 * i + 3] = m.nodes[i].w;
    }
    return JBGPU_OK;
}

int jbgpu_shape_local_inertia(const jbgpu_shape_desc* d, float mass, float out[3]) {
    if (!d || !out) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null argument");
    const float margin = 0.04f;
    switch (d->type) {
    case JBGPU_SHAPE_BOX: {       // BoxShape: dims = he - margin; calculateLocalInertia uses dims + margin
        float he[3];
        for (int k = 0; k < 3; k++) { volatile float dim = d->params[k] * 1.0f - margin; he[k] = dim + margin; }
        float lx = 2.0f * he[0], ly = 2.0f * he[1], lz = 2.0f * he[2];
        out[0] = mass / 12.0f * (ly * ly + lz * lz);
        out[1] = mass / 12.0f * (lx * lx + lz * lz);
        out[2] = mass / 12.0f * (lx * lx + ly * ly);
        return JBGPU_OK;
    }
    case JBGPU_SHAPE_SPHERE: {
        float r = d->params[0];
        float e = 0.4f * mass * r * r;
        out[0] = out[1] = out[2] = e;
        return JBGPU_OK;
    }
    case JBGPU_SHAPE_CAPSULE: {
        float r = d->params[0], hh = 0.5f * d->params[1];
        float he[3] = {r, r + hh, r};
        float lx = 2.0f * (he[0] + margin), ly = 2.0f * (he[1] + margin), lz = 2.0f * (he[2] + margin);
        float x2 = lx * lx, y2 = ly * ly, z2 = lz * lz, sm = mass * 0.08333333f;
        out[0] = sm * (y2 + z2); out[1] = sm * (x2 + z2); out[2] = sm * (x2 + y2);
        return JBGPU_OK;
    }
    case JBGPU_SHAPE_CONVEX_HULL: {
        if (!d->points || d->num_points <= 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "hull without points");
        float mx[3], mn[3];
        for (int i = 0; i < 3; i++) {
            float bp = -1e30f, bm = -1e30f, vp = 0, vm = 0;
            for (int k = 0; k < d->num_points; k++) {
                float x = d->points[3 * k + i];
                if (x > bp) { bp = x; vp = x; }
                if (-x > bm) { bm = -x; vm = x; }
            }
            mx[i] = vp + margin;
            mn[i] = vm - margin;
        }
        float lhe[3], lc[3], amin[3], amax[3], he[3];
        for (int i = 0; i < 3; i++) {
            lhe[i] = (mx[i] - mn[i]) * 0.5f + margin;
            lc[i] = (mx[i] + mn[i]) * 0.5f;
            amin[i] = lc[i] - lhe[i];
            amax[i] = lc[i] + lhe[i];
            he[i] = (amax[i] - amin[i]) * 0.5f;
        }
        float lx = 2.0f * (he[0] + margin), ly = 2.0f * (he[1] + margin), lz = 2.0f * (he[2] + margin);
        float x2 = lx * lx, y2 = ly * ly, z2 = lz * lz, sm = mass * 0.08333333f;
        out[0] = (y2 + z2) * sm; out[1] = (x2 + z2) * sm; out[2] = (x2 + y2) * sm;
        return JBGPU_OK;
    }
    case JBGPU_SHAPE_STATIC_PLANE:
    case JBGPU_SHAPE_TRIANGLE_MESH:   // TriangleMeshShape.calculateLocalInertia: zero (static meshes)
        out[0] = out[1] = out[2] = 0.0f;
        return JBGPU_OK;
    case JBGPU_SHAPE_COMPOUND: {      // CompoundShape.calculateLocalInertia: the box of getAabb(identity)
        if (!d->children || !d->child_transforms || d->num_children <= 0 || d->num_children > JBGPU_COMPOUND_MAX_CHILDREN)
            return fail(JBGPU_ERR_INVALID_ARGUMENT, "a compound needs 1 .. JBGPU_COMPOUND_MAX_CHILDREN children");
        std::vector<float4> pts;   // the children's hull points (unused here)
        std::vector<HostShape> ch(d->num_children);
        for (int c = 0; c < d->num_children; c++) {
            int rc = convex_record(pts, d->children[c], ch[c]);
            if (rc) return rc;
        }
        float lmin[3], lmax[3], he[3];
        compound_local_aabb(ch, d->child_transforms, d->num_children, lmin, lmax);
        for (int k = 0; k < 3; k++) {
            float lhe = (lmax[k] - lmin[k]) * 0.5f;
            lhe = lhe + d->params[0];
            const float lc = (lmax[k] + lmin[k]) * 0.5f;
            const float c = lc * 1.0f + 0.0f;   // the identity transform's centre (libGDX mul: x*1 + y*0 + z*0)
            const float amin = c - lhe, amax = c + lhe;
            he[k] = (amax - amin) * 0.5f;
        }
        const float lx = 2.0f * he[0], ly = 2.0f * he[1], lz = 2.0f * he[2];
        out[0] = mass / 12.0f * (ly * ly + lz * lz);
        out[1] = mass / 12.0f * (lx * lx + lz * lz);
        out[2] = mass / 12.0f * (lx * lx + ly * ly);
        return JBGPU_OK;
    }
    }
    return fail(JBGPU_ERR_INVALID_ARGUMENT, "unknown shape type");
}

int jbgpu_world_create(const jbgpu_config* cfg, jbgpu_world** out) {
    if (!out) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null out");
    *out = nullptr;
    jbgpu_config c;
    if (cfg) c = *cfg; else jbgpu_config_default(&c);
    if (c.solver_mode & JBGPU_SOLVER_RANDMIZE_ORDER)
        return fail(JBGPU_ERR_UNSUPPORTED, "SOLVER_RANDMIZE_ORDER: the solver order is the colour order");
    if (!(c.solver_mode & JBGPU_SOLVER_CACHE_FRIENDLY))
        return fail(JBGPU_ERR_UNSUPPORTED, "only the cache-friendly solver path is implemented");
    if (c.num_iterations < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "num_iterations < 0");
    if (c.solver_parts < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "solver_parts < 0");
    if (c.solver_smem_bodies < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "solver_smem_bodies < 0");
    if (c.broadphase_rebuild_interval < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "broadphase_rebuild_interval < 0");
    if (c.solver_threads != 0 && c.solver_threads != 64 && c.solver_threads != 128 && c.solver_threads != 256)
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "solver_threads must be 0, 64, 128 or 256");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(JBGPU_ERR_NO_DEVICE, "no CUDA device");
    if (c.device < 0 || c.device >= ndev) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad device ordinal");
    jbgpu_world* w = new jbgpu_world();
    w->cfg = c;
    w->device = c.device;
    if (cudaSetDevice(w->device) != cudaSuccess) { delete w; return fail(JBGPU_ERR_CUDA, "cudaSetDevice"); }
    w->sms = num_sms_of(w->device);
    if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&w->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->evFork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->evJoin, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&w->evT0) != cudaSuccess || cudaEventCreate(&w->evT1) != cudaSuccess) {
        jbgpu_world_destroy(w);
        return fail(JBGPU_ERR_CUDA, "stream");
    }
    DevWorld& d = w->dw;
    for (int k = 0; k < 3; k++) d.gravityAcc[k] = c.gravity[k];
    d.cbt = c.contact_breaking_threshold;
    d.deactTime = c.deactivation_time;
    d.disableDeact = c.disable_deactivation;
    d.numIter = c.num_iterations;
    w->bb.rebuildInterval = std::max(1, c.broadphase_rebuild_interval);
    w->graphOn = c.step_graphs != 0;
    d.resTol = c.solver_residual > 0.0f ? c.solver_residual : 0.0f;
    d.maxIter = c.solver_max_iterations > 0 ? c.solver_max_iterations : 200;
    d.resScope = c.solver_residual_scope != 0 ? 1 : 0;
    d.erp = c.erp;
    d.warm = c.warmstarting_factor;
    d.slop = c.linear_slop;
    d.solverMode = c.solver_mode;
    int rc;
    if (cudaMalloc(&d.ctr, sizeof(int) * C_NCTR) != cudaSuccess || cudaMemset(d.ctr, 0, sizeof(int) * C_NCTR) != cudaSuccess ||
        cudaMallocHost(&w->hostPinned, sizeof(int) * 64) != cudaSuccess) {
        delete w;
        return fail(JBGPU_ERR_CUDA, "counter allocation");
    }
    SolverBuffers& S = w->sb;
    if ((rc = [&]() -> int {
             CK(dalloc(&S.colourCount, MAX_COLOURS + 1)); CK(dalloc(&S.colourFill, MAX_COLOURS + 1));
             CK(dalloc(&S.colourStart, MAX_COLOURS + 1)); CK(dalloc(&S.nCand, 1)); CK(dalloc(&S.nColours, 1));
             CK(dalloc(&S.nIslChunks, 1));
             CK(dalloc(&w->rows.nPts, 1));
             CK(cudaMemset(w->rows.nPts, 0, sizeof(int)));
             CK(cudaMemset(S.nCand, 0, sizeof(int))); CK(cudaMemset(S.nColours, 0, sizeof(int)));
             NarrowBuffers& N = w->nb;
             N.slots = w->sms * 2;
             if (narrowphase_configure()) return fail(JBGPU_ERR_CUDA, "EPA shared-memory size");
             CK(dalloc(&N.queueCount, 1));
             CK(dalloc(&N.ovfCount, 3));
             CK(cudaMemset(N.ovfCount, 0, sizeof(int) * 3));

             return grow_bodies(w, std::max(1, c.initial_body_capacity));
         }()) != JBGPU_OK) {
        jbgpu_world_destroy(w);
        return rc;
    }
    *out = w;
    return JBGPU_OK;
}

int jbgpu_world_destroy(jbgpu_world* w) {
    if (!w) return JBGPU_OK;
    cudaSetDevice(w->device);
    if (w->stream) cudaStreamSynchronize(w->stream);
    if (w->aux) cudaStreamSynchronize(w->aux);
    graphs_clear(w);
    query_free(w->qb);
    DevWorld& d = w->dw;
    dfree(d.xr0); dfree(d.xr1); dfree(d.xr2); dfree(d.kx0); dfree(d.kx1); dfree(d.kx2); dfree(d.ilv); dfree(d.iav); dfree(d.hitf); dfree(d.linvel); dfree(d.angvel); dfree(d.iw0); dfree(d.iw1); dfree(d.iw2);
    dfree(d.iloc); dfree(d.force); dfree(d.torque); dfree(d.gravity); dfree(d.amin); dfree(d.amax); dfree(d.act);
    dfree(d.deact); dfree(d.flags); dfree(d.shape); dfree(d.group); dfree(d.mask); dfree(d.world); dfree(d.friction);
    dfree(d.restitution); dfree(d.linSleep); dfree(d.angSleep); dfree(d.linDamp); dfree(d.angDamp); dfree(d.island);
    dfree(d.ccdThr); dfree(d.ccdRad);
    ccd_free(w->cb);
    dfree(d.ctr);
    DevShapes& S = d.sh;
    dfree(S.type); dfree(S.margin); dfree(S.dims); dfree(S.laabb_min); dfree(S.laabb_max); dfree(S.plane);
    dfree(S.hull_off); dfree(S.hull_cnt); dfree(S.hull_pts);
    dfree(S.child_off); dfree(S.child_cnt); dfree(S.child_shape); dfree(S.child_xf); dfree(S.mesh_node_off);
    dfree(S.mesh_node_cnt); dfree(S.mesh_tri_off); dfree(S.mesh_q); dfree(S.mesh_nodes); dfree(S.mesh_tris);
    concave_free(w->nb);
    free_pairs(w->pairs[0]);
    free_pairs(w->pairs[1]);
    DevRows& R = w->rows;
    dfree(R.n_nrm); dfree(R.n_rp1); dfree(R.n_rp2); dfree(R.n_angA); dfree(R.n_angB);
    dfree(R.f_nrm); dfree(R.f_rp1); dfree(R.f_rp2); dfree(R.f_angA); dfree(R.f_angB);
    dfree(R.slot_pair); dfree(R.slot_desc); dfree(R.slot_im); dfree(R.slot_pt0); dfree(R.pt_key); dfree(R.nPts);
    BroadphaseBuffers& B = w->bb;
    dfree(B.bounds); dfree(B.mkeys); dfree(B.mkeys_alt); dfree(B.sortedBody); dfree(B.vals_alt);
    if (B.sortScratch) cudaFree(B.sortScratch);
    if (B.scanScratch) cudaFree(B.scanScratch);
    dfree(B.bvh.left); dfree(B.bvh.right); dfree(B.bvh.lo); dfree(B.bvh.hi); dfree(B.bvh.parent); dfree(B.bvh.leafParent);
    dfree(B.bvh.visit); dfree(B.bvh.node); dfree(B.tcount); dfree(B.tcache); dfree(B.wstart); dfree(B.wend); dfree(B.wroot);
    dfree(B.planeList); dfree(B.planeStart); dfree(B.cnt); dfree(B.off); dfree(B.offPrev); dfree(B.cursor); dfree(B.total); dfree(B.partners);
    dfree(B.candBound); dfree(B.segLong);
    NarrowBuffers& N = w->nb;
    if (N.queue) cudaFree(N.queue);
    dfree(N.queueCount); dfree(N.ovfQueue); dfree(N.ovfQueue2); dfree(N.ovfCount); dfree(N.pairBucket); dfree(N.perm); dfree(N.blockOff);
    if (N.scanScratch) cudaFree(N.scanScratch);
    SolverBuffers& V = w->sb;
    dfree(V.parent); dfree(V.keepAwake); dfree(V.inactive); dfree(V.flag); dfree(V.candIdx); dfree(V.cand); dfree(V.colourOf);
    dfree(V.bucket); dfree(V.bucketList); dfree(V.claim); dfree(V.taken); dfree(V.posOf); dfree(V.candLocal);
    dfree(V.md); dfree(V.ml); dfree(V.slotIsl); dfree(V.islList); dfree(V.islCount); dfree(V.islFill); dfree(V.islStart);
    dfree(V.segFlag); dfree(V.segIdx); dfree(V.islChunk); dfree(V.islConv); dfree(V.islAcc); dfree(V.islDone);
    dfree(V.resTrace);
    {
        DevJoints& J = V.J;
        dfree(J.a); dfree(J.b); dfree(J.pivA); dfree(J.pivB); dfree(J.set); dfree(J.order); dfree(J.colStart);
        dfree(J.r1); dfree(J.r2); dfree(J.dep); dfree(J.imp); dfree(J.act);
        dfree(J.kind); dfree(J.set2); dfree(J.frame); dfree(J.hs); dfree(J.d6set);
    }
    dfree(V.nIslChunks);
    if (V.islScratch) cudaFree(V.islScratch);
    dfree(V.colourCount); dfree(V.colourFill); dfree(V.colourStart);
    solver_free(V);
    dfree(V.nCand); dfree(V.nColours);
    if (V.scanScratch) cudaFree(V.scanScratch);
    if (w->hostPinned) cudaFreeHost(w->hostPinned);
    free_prof(w->prof);
    if (w->profHist) cudaFree(w->profHist);
    if (w->ioStage) cudaFree(w->ioStage);
    dfree(w->sampleX);
    dfree(w->sampleT);
    if (w->evFork) cudaEventDestroy(w->evFork);
    if (w->evJoin) cudaEventDestroy(w->evJoin);
    if (w->evT0) cudaEventDestroy(w->evT0);
    if (w->evT1) cudaEventDestroy(w->evT1);
    if (w->aux) cudaStreamDestroy(w->aux);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
    return JBGPU_OK;
}

int jbgpu_world_add_shapes(jbgpu_world* w, const jbgpu_shape_desc* shapes, int32_t n, int32_t* ids) {
    if (!w || (!shapes && n > 0) || n < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad arguments");
    for (int i = 0; i < n; i++) {
        const jbgpu_shape_desc& d = shapes[i];
        HostShape h;
        std::memset(&h, 0, sizeof(h));
        h.type = d.type;
        h.margin = 0.04f;
        switch (d.type) {
        case JBGPU_SHAPE_BOX:
        case JBGPU_SHAPE_SPHERE:
        case JBGPU_SHAPE_CAPSULE:
        case JBGPU_SHAPE_CONVEX_HULL: {
            int rc = convex_record(w->hullPts, d, h);
            if (rc) return rc;
            break;
        }
        case JBGPU_SHAPE_STATIC_PLANE: {   // normal.nor() (libGDX: skipped when len2 is 0 or 1)
            float x = d.params[0], y = d.params[1], z = d.params[2];
            float l2 = x * x + y * y + z * z;
            if (!(l2 == 0.0f || l2 == 1.0f)) {
                float s = 1.0f / std::sqrt(l2);
                x = x * s; y = y * s; z = z * s;
            }
            h.plane[0] = x; h.plane[1] = y; h.plane[2] = z; h.plane[3] = d.params[3];
            break;
        }
        case JBGPU_SHAPE_TRIANGLE_MESH: {   // BvhTriangleMeshShape(TriangleIndexVertexArray, true),
                                            // setLocalScaling, setMargin
            MeshBvh m;
            std::vector<float> scaled;
            if (build_mesh_bvh(mesh_vertices(d, scaled), d.num_points, d.indices, d.num_triangles, m))
                return fail(JBGPU_ERR_INVALID_ARGUMENT, "a triangle mesh needs vertices, 1 .. 2^21-1 triangles and "
                                                        "indices within the vertex array");
            h.margin = d.params[0];
            h.node_off = (int)w->meshNodes.size();
            h.node_cnt = (int)m.nodes.size();
            h.tri_off = (int)(w->meshTris.size() / 3);
            MeshSource src;   // what a refit of this mesh needs
            src.shape = (int)w->shapes.size();
            src.numPoints = d.num_points;
            src.idx.assign(d.indices, d.indices + (size_t)3 * d.num_triangles);
            for (int k = 0; k < 3; k++) src.scaling[k] = d.params[1 + k];
            w->meshSrc.push_back(std::move(src));
            w->meshNodes.insert(w->meshNodes.end(), m.nodes.begin(), m.nodes.end());
            w->meshTris.insert(w->meshTris.end(), m.tris.begin(), m.tris.end());
            for (int k = 0; k < 3; k++) {
                h.lmin[k] = m.lmin[k]; h.lmax[k] = m.lmax[k];
                h.q[k] = m.bmin[k]; h.q[4 + k] = m.bmax[k]; h.q[8 + k] = m.quant[k];
            }
            w->hasMesh = true;
            break;
        }
        case JBGPU_SHAPE_COMPOUND: {
            if (!d.children || !d.child_transforms || d.num_children <= 0 || d.num_children > JBGPU_COMPOUND_MAX_CHILDREN)
                return fail(JBGPU_ERR_INVALID_ARGUMENT, "a compound needs 1 .. JBGPU_COMPOUND_MAX_CHILDREN children");
            std::vector<HostShape> ch(d.num_children);
            for (int c = 0; c < d.num_children; c++) {
                int rc = convex_record(w->hullPts, d.children[c], ch[c]);
                if (rc) return rc;
            }
            compound_local_aabb(ch, d.child_transforms, d.num_children, h.lmin, h.lmax);
            h.margin = d.params[0];
            h.child_off = (int)w->childShapes.size();
            h.child_cnt = d.num_children;
            for (int c = 0; c < d.num_children; c++) {
                const float* t = d.child_transforms + 12 * c;
                w->childShapes.push_back(ch[c]);
                w->childXf.push_back(make_float4(t[0], t[1], t[2], t[9]));
                w->childXf.push_back(make_float4(t[3], t[4], t[5], t[10]));
                w->childXf.push_back(make_float4(t[6], t[7], t[8], t[11]));
            }
            w->hasCompound = true;
            break;
        }
        default:
            return fail(JBGPU_ERR_UNSUPPORTED, "shape type not on this path");
        }
        if (ids) ids[i] = (int)w->shapes.size();
        w->shapes.push_back(h);
    }
    w->shapesDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_add_shape(jbgpu_world* w, const jbgpu_shape_desc* s, int32_t* id) { return jbgpu_world_add_shapes(w, s, 1, id); }

int jbgpu_world_refit_mesh(jbgpu_world* w, int32_t shape, const float* points, int32_t num_points) {
    if (!w || !points || shape < 0 || shape >= (int)w->shapes.size() || w->shapes[shape].type != JBGPU_SHAPE_TRIANGLE_MESH)
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "refit_mesh: a triangle-mesh shape id and its vertices");
    const MeshSource* src = nullptr;
    for (const MeshSource& m : w->meshSrc)
        if (m.shape == shape) src = &m;
    if (!src || num_points != src->numPoints)
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "refit_mesh: the vertex count differs from the shape's");
    HostShape& h = w->shapes[shape];
    const int nt = (int)src->idx.size() / 3;
    std::vector<float> buf;
    const float* v = scaled_vertices(points, num_points, src->scaling, buf);
    MeshBvh m;
    m.nodes.assign(w->meshNodes.begin() + h.node_off, w->meshNodes.begin() + h.node_off + h.node_cnt);
    m.tris.resize((size_t)3 * nt);
    refit_mesh_bvh(v, src->idx.data(), nt, h.margin, m);
    std::copy(m.nodes.begin(), m.nodes.end(), w->meshNodes.begin() + h.node_off);
    std::copy(m.tris.begin(), m.tris.end(), w->meshTris.begin() + (size_t)3 * h.tri_off);
    for (int k = 0; k < 3; k++) {
        h.lmin[k] = m.lmin[k]; h.lmax[k] = m.lmax[k];
        h.q[k] = m.bmin[k]; h.q[4 + k] = m.bmax[k]; h.q[8 + k] = m.quant[k];
    }
    w->shapesDirty = true;
    w->aabbRefresh.push_back(shape);
    return JBGPU_OK;
}

int jbgpu_world_mesh_bvh(const jbgpu_world* w, int32_t shape, int32_t* nodes, int32_t capacity, int32_t* n,
                         float aabb[6]) {
    if (!w || !n || shape < 0 || shape >= (int)w->shapes.size() || w->shapes[shape].type != JBGPU_SHAPE_TRIANGLE_MESH ||
        capacity < 0 || (capacity > 0 && !nodes))
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "mesh_bvh: a triangle-mesh shape id, a count pointer and a node buffer");
    const HostShape& h = w->shapes[shape];
    *n = h.node_cnt;
    if (aabb)
        for (int k = 0; k < 3; k++) { aabb[k] = h.lmin[k]; aabb[3 + k] = h.lmax[k]; }
    if (h.node_cnt > capacity) return fail(JBGPU_ERR_CAPACITY, "node buffer too small");
    for (int i = 0; i < h.node_cnt; i++) {
        const int4 q = w->meshNodes[h.node_off + i];
        nodes[4 * i] = q.x; nodes[4 * i + 1] = q.y; nodes[4 * i + 2] = q.z; nodes[4 * i + 3] = q.w;
    }
    return JBGPU_OK;
}

int jbgpu_world_num_bodies(const jbgpu_world* w, int32_t* n) {
    if (!w || !n) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    *n = w->nBodies;
    return JBGPU_OK;
}

int jbgpu_world_add_bodies(jbgpu_world* w, const jbgpu_body_desc* b, int32_t n, int32_t* uids) {
    if (!w || (!b && n > 0) || n < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad arguments");
    if (n == 0) return JBGPU_OK;
    if ((long long)w->nBodies + n > MAX_BODIES_KEYED) return fail(JBGPU_ERR_CAPACITY, "pair keys hold body indices below 2^24");
    CK(cudaSetDevice(w->device));
    for (int i = 0; i < n; i++) {
        if (b[i].shape < 0 || b[i].shape >= (int)w->shapes.size()) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad shape id");
        if (w->shapes[b[i].shape].type == JBGPU_SHAPE_STATIC_PLANE && b[i].mass != 0.0f)
            return fail(JBGPU_ERR_INVALID_ARGUMENT, "a static plane must have mass 0");
        if (w->shapes[b[i].shape].type == JBGPU_SHAPE_TRIANGLE_MESH && b[i].mass != 0.0f)
            return fail(JBGPU_ERR_INVALID_ARGUMENT, "a triangle mesh body must have mass 0 (moving concave objects are "
                                                    "not supported, TriangleMeshShape.calculateLocalInertia)");
        if (b[i].world < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "negative world index");
        if (b[i].collision_flags & ~(1 | JBGPU_CF_KINEMATIC_OBJECT | JBGPU_CF_NO_CONTACT_RESPONSE))
            return fail(JBGPU_ERR_UNSUPPORTED, "collision flags other than KINEMATIC_OBJECT and NO_CONTACT_RESPONSE");
        if (b[i].activation_state < 0 || b[i].activation_state > JBGPU_DISABLE_SIMULATION)
            return fail(JBGPU_ERR_INVALID_ARGUMENT, "activation state outside 0 .. DISABLE_SIMULATION");
    }
    int rc = grow_bodies(w, w->nBodies + n);
    if (rc) return rc;
    w->bb.offPrevValid = false;   // last step's per-owner offsets cover the old bodies only
    rc = sync_shapes(w);
    if (rc) return rc;
    std::vector<float4> xr0(n), xr1(n), xr2(n), lv(n), av(n), iloc(n), grav(n), zero(n, make_float4(0, 0, 0, 0));
    std::vector<int> act(n, JBGPU_ACTIVE_TAG), flags(n), shape(n), group(n), mask(n), world(n);
    std::vector<float> deact(n, 0.0f), fr(n), re(n), ls(n), as(n), ld(n), ad(n);
    for (int i = 0; i < n; i++) {
        const jbgpu_body_desc& d = b[i];
        const float* t = d.transform;
        xr0[i] = make_float4(t[0], t[1], t[2], t[9]);
        xr1[i] = make_float4(t[3], t[4], t[5], t[10]);
        xr2[i] = make_float4(t[6], t[7], t[8], t[11]);
        lv[i] = make_float4(d.linear_velocity[0], d.linear_velocity[1], d.linear_velocity[2], 0);
        av[i] = make_float4(d.angular_velocity[0], d.angular_velocity[1], d.angular_velocity[2], 0);
        int f = d.collision_flags & (CF_KINEMATIC | CF_NO_CONTACT_RESPONSE);
        if (f & CF_KINEMATIC) w->hasKinematic = true;
        if (d.activation_state != 0) act[i] = d.activation_state;
        float im;
        if (d.mass == 0.0f) { f |= CF_STATIC; im = 0.0f; } else im = 1.0f / d.mass;
        if (w->shapes[d.shape].type == JBGPU_SHAPE_STATIC_PLANE || w->shapes[d.shape].type == JBGPU_SHAPE_TRIANGLE_MESH)
            f |= CF_LISTED;
        float il[3];
        for (int k = 0; k < 3; k++) il[k] = d.local_inertia[k] != 0.0f ? 1.0f / d.local_inertia[k] : 0.0f;
        iloc[i] = make_float4(il[0], il[1], il[2], im);
        float g[3] = {0, 0, 0};
        if (!(f & (CF_STATIC | CF_KINEMATIC)) && im != 0.0f) {
            float inv = 1.0f / im;
            for (int k = 0; k < 3; k++) g[k] = w->cfg.gravity[k] * inv;
        }
        grav[i] = make_float4(g[0], g[1], g[2], 0);
        bool dynamic = !(f & (CF_STATIC | CF_KINEMATIC));
        group[i] = d.collision_group != -1 ? (int)(short)d.collision_group : (dynamic ? 1 : 2);
        mask[i] = d.collision_mask != -1 ? (int)(short)d.collision_mask : (dynamic ? -1 : (int)(short)(-1 ^ 2));
        flags[i] = f;
        shape[i] = d.shape;
        world[i] = d.world;
        fr[i] = d.friction; re[i] = d.restitution; ls[i] = d.linear_sleeping_threshold; as[i] = d.angular_sleeping_threshold;
        auto clamp01 = [](float x) { return x < 0.0f ? 0.0f : (1.0f < x ? 1.0f : x); };
        ld[i] = clamp01(d.linear_damping);
        ad[i] = clamp01(d.angular_damping);
        w->hShape.push_back(d.shape);
        w->hWorld.push_back(d.world);
        w->hFlags.push_back(f);
        if (uids) uids[i] = w->nBodies + i + 1;
    }
    int o = w->nBodies;
    cudaStream_t s = w->stream;
    DevWorld& D = w->dw;
#define UP(dst, src, T) CK(cudaMemcpyAsync(D.dst + o, src.data(), sizeof(T) * n, cudaMemcpyHostToDevice, s))
    UP(xr0, xr0, float4); UP(xr1, xr1, float4); UP(xr2, xr2, float4); UP(linvel, lv, float4); UP(angvel, av, float4);
    UP(kx0, xr0, float4); UP(kx1, xr1, float4); UP(kx2, xr2, float4);   // interpolationWorldTransform = worldTransform
    UP(ilv, zero, float4); UP(iav, zero, float4);                          // interpolation velocities 0
    {
        const std::vector<float> one(n, 1.0f);                              // hitFraction 1
        UP(hitf, one, float);
    }
    UP(iloc, iloc, float4); UP(gravity, grav, float4); UP(force, zero, float4); UP(torque, zero, float4);
    UP(act, act, int); UP(deact, deact, float); UP(flags, flags, int); UP(shape, shape, int); UP(group, group, int);
    UP(mask, mask, int); UP(world, world, int); UP(friction, fr, float); UP(restitution, re, float);
    UP(linSleep, ls, float); UP(angSleep, as, float); UP(linDamp, ld, float); UP(angDamp, ad, float);
#undef UP
    w->nBodies += n;
    DevWorld dv = dev_view(w);
    k_init_bodies<<<(n + 255) / 256, 256, 0, s>>>(dv, o, n); note_launch();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    w->planesDirty = true;
    return JBGPU_OK;
}


int jbgpu_world_remove_bodies(jbgpu_world* w, const int32_t* bodies, int32_t n) {
    if (!w || n < 0 || (n > 0 && !bodies)) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad arguments");
    if (n == 0) return JBGPU_OK;
    const int nOld = w->nBodies;
    std::vector<int> newIndex(nOld, 0);
    for (int k = 0; k < n; k++) {
        if (bodies[k] < 0 || bodies[k] >= nOld) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad body index");
        if (newIndex[bodies[k]] < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "a body listed twice");
        newIndex[bodies[k]] = -1;
    }
    for (size_t j = 0; j < w->jA.size(); j++)
        if ((w->jA[j] >= 0 && newIndex[w->jA[j]] < 0) || (w->jB[j] >= 0 && newIndex[w->jB[j]] < 0))
            return fail(JBGPU_ERR_INVALID_ARGUMENT, "a joint uses a body to remove (remove the joint first)");
    std::vector<int> from;
    for (int i = 0; i < nOld; i++)
        if (newIndex[i] >= 0) { newIndex[i] = (int)from.size(); from.push_back(i); }
    const int nNew = (int)from.size();
    CK(cudaSetDevice(w->device));
    cudaStream_t s = w->stream;
    CK(cudaStreamSynchronize(s));
    int *dFrom = nullptr, *dNew = nullptr;
    void* tmp = nullptr;
    CK(dalloc(&dFrom, std::max(nNew, 1)));
    CK(dalloc(&dNew, nOld));
    CK(cudaMalloc(&tmp, sizeof(float4) * std::max(nNew, 1)));
    CK(cudaMemcpy(dFrom, from.data(), sizeof(int) * nNew, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dNew, newIndex.data(), sizeof(int) * nOld, cudaMemcpyHostToDevice));
    DevWorld& d = w->dw;
    int rc = 0;
    using namespace removal;
#define GA(ptr) if (!rc) rc = gather_array(d.ptr, dFrom, nNew, tmp, s)
    GA(xr0); GA(xr1); GA(xr2); GA(kx0); GA(kx1); GA(kx2); GA(ilv); GA(iav); GA(hitf); GA(linvel); GA(angvel); GA(iw0); GA(iw1); GA(iw2); GA(iloc);
    GA(force); GA(torque); GA(gravity); GA(amin); GA(amax); GA(act); GA(deact); GA(flags); GA(shape); GA(group);
    GA(mask); GA(world); GA(friction); GA(restitution); GA(linSleep); GA(angSleep); GA(linDamp); GA(angDamp);
    GA(ccdThr); GA(ccdRad);
#undef GA
    // the pairs of kept bodies, renumbered, into the other pair buffer
    const int np = w->nPairs;
    int kept = 0;
    if (!rc && np > 0) {
        const int nxt = w->cur ^ 1;
        rc = ensure_pair_capacity(w, nxt, np);
        int *flag = nullptr, *pos = nullptr, *tot = nullptr;
        void* scratch = nullptr;
        if (!rc && (dalloc(&flag, np) != cudaSuccess || dalloc(&pos, np) != cudaSuccess || dalloc(&tot, 1) != cudaSuccess ||
                    cudaMalloc(&scratch, scan_scratch_bytes(np)) != cudaSuccess))
            rc = fail(JBGPU_ERR_CUDA, "pair compaction buffers");
        if (!rc) {
            k_pairs_keep<<<(np + 255) / 256, 256, 0, s>>>(w->pairs[w->cur], np, dNew, flag); note_launch();
            exclusive_scan(flag, pos, tot, np, scratch, s);
            k_pairs_move<<<(np + 255) / 256, 256, 0, s>>>(w->pairs[w->cur], w->pairs[nxt], np, flag, pos, dNew);
            note_launch();
            // the device's pair count (which the replayed step reads as last step's) follows
            if (cudaMemcpyAsync(w->dw.ctr + C_PAIRS, tot, sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(&kept, tot, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)
                rc = fail(JBGPU_ERR_CUDA, "pair compaction");
            else
                w->cur = nxt;
        }
        dfree(flag); dfree(pos); dfree(tot);
        if (scratch) cudaFree(scratch);
    }
    if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = fail(JBGPU_ERR_CUDA, "body compaction");
    dfree(dFrom); dfree(dNew);
    cudaFree(tmp);
    if (rc) return rc;
    w->nPairs = kept;
    auto compact = [&](std::vector<int>& v) {
        std::vector<int> o(nNew);
        for (int j = 0; j < nNew; j++) o[j] = v[from[j]];
        v.swap(o);
    };
    compact(w->hShape); compact(w->hWorld); compact(w->hFlags);
    for (size_t j = 0; j < w->jA.size(); j++) {   // the joints' bodies renumbered
        if (w->jA[j] >= 0) w->jA[j] = newIndex[w->jA[j]];
        if (w->jB[j] >= 0) w->jB[j] = newIndex[w->jB[j]];
    }
    if (!w->jA.empty()) w->jointsDirty = true;
    w->nBodies = nNew;
    w->bb.offPrevValid = false;
    w->planesDirty = true;   // listed bodies, per-world counts, the tree and the solver parts
    graphs_clear(w);
    return JBGPU_OK;
}

int jbgpu_world_step(jbgpu_world* w, float dt, int32_t substeps) {
    if (!w || substeps < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad arguments");
    if (w->inTick) return fail(JBGPU_ERR_INVALID_ARGUMENT, "a tick callback cannot step the world");
    int rc = prepare(w);
    if (rc) return rc;
    CK(cudaMemsetAsync(w->dw.ctr + C_STATUS, 0, sizeof(int), w->stream));
    if (w->hasKinematic && (rc = run_stage(w, JBGPU_STAGE_SAVE_KINEMATIC, dt))) return rc;
    if ((rc = run_stage(w, JBGPU_STAGE_APPLY_GRAVITY, dt))) return rc;
    for (int i = 0; i < substeps; i++)
        if ((rc = single_step(w, dt)) || (rc = bodyprops::after_substep(w, dt))) return rc;
    if ((rc = run_stage(w, JBGPU_STAGE_CLEAR_FORCES, dt))) return rc;
    return check_status(w);
}

int jbgpu_world_step_simulation(jbgpu_world* w, float timeStep, int32_t maxSubSteps, float fixedTimeStep, int32_t* numOut) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    if (w->inTick) return fail(JBGPU_ERR_INVALID_ARGUMENT, "a tick callback cannot step the world");
    int num = 0;
    if (maxSubSteps != 0) {
        w->localTime += timeStep;
        if (w->localTime >= fixedTimeStep) {
            num = (int)(w->localTime / fixedTimeStep);
            w->localTime -= num * fixedTimeStep;
        }
    } else {
        fixedTimeStep = timeStep;
        w->localTime = timeStep;
        if (std::fabs(timeStep) < 1.19209290e-07f) { num = 0; maxSubSteps = 0; }
        else { num = 1; maxSubSteps = 1; }
    }
    if (numOut) *numOut = num;
    int rc = prepare(w);
    if (rc) return rc;
    CK(cudaMemsetAsync(w->dw.ctr + C_STATUS, 0, sizeof(int), w->stream));
    if (num != 0) {
        if (w->hasKinematic && (rc = run_stage(w, JBGPU_STAGE_SAVE_KINEMATIC, fixedTimeStep))) return rc;
        if ((rc = run_stage(w, JBGPU_STAGE_APPLY_GRAVITY, fixedTimeStep))) return rc;
        int clamped = num > maxSubSteps ? maxSubSteps : num;
        for (int i = 0; i < clamped; i++)
            if ((rc = single_step(w, fixedTimeStep)) || (rc = bodyprops::after_substep(w, fixedTimeStep))) return rc;
    }
    if ((rc = run_stage(w, JBGPU_STAGE_CLEAR_FORCES, fixedTimeStep))) return rc;
    return check_status(w);
}

int jbgpu_world_stage(jbgpu_world* w, int32_t stage, float dt) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    if (w->inTick) return fail(JBGPU_ERR_INVALID_ARGUMENT, "a tick callback cannot step the world");
    int rc = prepare(w);
    if (rc) return rc;
    CK(cudaMemsetAsync(w->dw.ctr + C_STATUS, 0, sizeof(int), w->stream));
    if ((rc = run_stage(w, stage, dt))) return rc;
    return check_status(w);
}

// The narrowphase stage with the EPA scratch compiled into the library: no device or host
// allocation on this path (the lookup of the scratch address, once per device, allocates
// nothing either).  Shapes or bodies added since the last step or stage would be uploaded by
// an allocating path, so they are refused here instead.
int jbgpu_world_narrowphase_static(jbgpu_world* w, int32_t epa_slots) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    if (epa_slots <= 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "epa_slots must be positive");
    if (epa_slots > JBGPU_STATIC_EPA_SLOTS_MAX)
        return fail(JBGPU_ERR_CAPACITY, "epa_slots exceeds the static EPA scratch (JBGPU_STATIC_EPA_SLOTS_MAX = 32)");
    if (w->shapesDirty || w->planesDirty)
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "shapes or bodies added since the last step or stage: run one first");
    if (w->hasMesh)
        return fail(JBGPU_ERR_UNSUPPORTED, "the static-scratch narrowphase does not run the triangle-mesh pass");
    if (w->device >= MAX_STATIC_DEVICES) return fail(JBGPU_ERR_UNSUPPORTED, "device ordinal beyond the static scratch table");
    CK(cudaSetDevice(w->device));
    void* base = nullptr;
    if (epa_static_scratch(w->device, &base)) return fail(JBGPU_ERR_CUDA, "cudaGetSymbolAddress of the static EPA scratch");
    cudaStream_t s = w->stream;
    CK(cudaMemsetAsync(w->dw.ctr + C_STATUS, 0, sizeof(int), s));
    CK(cudaMemsetAsync(w->dw.ctr + C_GJK, 0, sizeof(int) * 2, s));
    narrowphase_launch_static(dev_view(w), w->pairs[w->cur], w->nPairs, w->nb, base, epa_slots, s);
    CK(cudaGetLastError());
    return check_status(w);
}

int jbgpu_world_set_ccd(jbgpu_world* w, const int32_t* bodies, const float* thr, const float* rad, int32_t n) {
    if (!w || n < 0 || (n > 0 && (!bodies || !thr || !rad))) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad CCD arguments");
    for (int k = 0; k < n; k++)
        if (bodies[k] < 0 || bodies[k] >= w->nBodies) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad body index");
    if (n == 0) return JBGPU_OK;
    CK(cudaSetDevice(w->device));
    CK(cudaStreamSynchronize(w->stream));
    std::vector<float> t(w->nBodies), r(w->nBodies);
    CK(cudaMemcpy(t.data(), w->dw.ccdThr, sizeof(float) * w->nBodies, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r.data(), w->dw.ccdRad, sizeof(float) * w->nBodies, cudaMemcpyDeviceToHost));
    for (int k = 0; k < n; k++) {
        t[bodies[k]] = thr[k];
        r[bodies[k]] = rad[k];
    }
    CK(cudaMemcpy(w->dw.ccdThr, t.data(), sizeof(float) * w->nBodies, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w->dw.ccdRad, r.data(), sizeof(float) * w->nBodies, cudaMemcpyHostToDevice));
    bool on = false;
    for (float v : t) on = on || v != 0.0f;
    if (on != w->ccdOn) graphs_clear(w);   // the integrate stage's launches change
    w->ccdOn = on;
    return JBGPU_OK;
}

// RigidBody.setGravity on the host copy of the bodies' inverse masses and gravity forces:
// gravity = acceleration * (1 / inverseMass) for inverseMass != 0 (binary32, no contraction).
static int body_gravity(jbgpu_world* w, const int32_t* bodies, const float* acc, int32_t n, bool all) {
    if (w->nBodies == 0) return JBGPU_OK;
    CK(cudaSetDevice(w->device));
    CK(cudaStreamSynchronize(w->stream));
    std::vector<float4> il(w->nBodies), g(w->nBodies);
    CK(cudaMemcpy(il.data(), w->dw.iloc, sizeof(float4) * w->nBodies, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(g.data(), w->dw.gravity, sizeof(float4) * w->nBodies, cudaMemcpyDeviceToHost));
    const int m = all ? w->nBodies : n;
    for (int k = 0; k < m; k++) {
        const int i = all ? k : bodies[k];
        const float* a = all ? acc : acc + 3 * k;
        const float im = il[i].w;
        if (im != 0.0f) {
            const float s = 1.0f / im;
            g[i] = make_float4(a[0] * s, a[1] * s, a[2] * s, 0.0f);
        }
    }
    CK(cudaMemcpy(w->dw.gravity, g.data(), sizeof(float4) * w->nBodies, cudaMemcpyHostToDevice));
    return JBGPU_OK;
}

int jbgpu_world_apply_impulses(jbgpu_world* w, const int32_t* bodies, const float* imp, const float* rel, const float* tq,
                               int32_t n) {
    if (!w || n < 0 || (n > 0 && (!bodies || (!imp && !tq)))) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad impulse arguments");
    if (n == 0) return JBGPU_OK;
    if (int rc = bodyprops::check_distinct(w, bodies, n)) return rc;
    CK(cudaSetDevice(w->device));
    cudaStream_t s = w->stream;
    int* dB = nullptr;
    float* dF = nullptr;
    CK(dalloc(&dB, n));
    CK(dalloc(&dF, (size_t)9 * n));
    CK(cudaMemcpyAsync(dB, bodies, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    float* dI = imp ? dF : nullptr;
    float* dR = rel ? dF + 3 * n : nullptr;
    float* dT = tq ? dF + 6 * n : nullptr;
    if (imp) CK(cudaMemcpyAsync(dI, imp, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
    if (rel) CK(cudaMemcpyAsync(dR, rel, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
    if (tq) CK(cudaMemcpyAsync(dT, tq, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
    launch_apply_impulses(dev_view(w), dB, dI, dR, dT, n, s);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    dfree(dB);
    dfree(dF);
    return JBGPU_OK;
}

int jbgpu_world_set_body_properties(jbgpu_world* w, const int32_t* bodies, int32_t n, const float* linear_damping,
                                    const float* angular_damping, const float* friction, const float* restitution,
                                    const float* linear_sleeping_threshold, const float* angular_sleeping_threshold) {
    if (!w || n < 0 || (n > 0 && !bodies)) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad body property arguments");
    if (n == 0) return JBGPU_OK;
    if (int rc = bodyprops::check_distinct(w, bodies, n)) return rc;
    const float* src[6] = {linear_damping, angular_damping, friction, restitution, linear_sleeping_threshold,
                           angular_sleeping_threshold};
    float* dst[6] = {w->dw.linDamp, w->dw.angDamp, w->dw.friction, w->dw.restitution, w->dw.linSleep, w->dw.angSleep};
    std::vector<float> host((size_t)6 * n);
    int m = 0;
    for (int q = 0; q < 6; q++) {
        if (!src[q]) continue;
        for (int k = 0; k < n; k++) {
            float x = src[q][k];
            if (q < 2) x = x < 0.0f ? 0.0f : (1.0f < x ? 1.0f : x);   // RigidBody.setDamping: MiscUtil.GEN_clamped to [0, 1]
            host[(size_t)m * n + k] = x;
        }
        m++;
    }
    if (m == 0) return JBGPU_OK;
    CK(cudaSetDevice(w->device));
    cudaStream_t s = w->stream;
    int* dB = nullptr;
    float* dV = nullptr;
    CK(dalloc(&dB, n));
    CK(dalloc(&dV, (size_t)m * n));
    CK(cudaMemcpyAsync(dB, bodies, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dV, host.data(), sizeof(float) * m * n, cudaMemcpyHostToDevice, s));
    for (int q = 0, j = 0; q < 6; q++) {
        if (!src[q]) continue;
        bodyprops::k_scatter<<<(n + 127) / 128, 128, 0, s>>>(dst[q], dB, dV + (size_t)j * n, n);
        note_launch();
        j++;
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    dfree(dB);
    dfree(dV);
    return JBGPU_OK;
}

int jbgpu_world_set_internal_tick_callback(jbgpu_world* w, jbgpu_tick_callback cb, void* user) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    if (w->inTick) return fail(JBGPU_ERR_INVALID_ARGUMENT, "the tick callback cannot be replaced from inside it");
    w->tickCb = cb;
    w->tickUser = cb ? user : nullptr;
    return JBGPU_OK;
}

int jbgpu_world_set_gravity(jbgpu_world* w, const float gravity[3]) {
    if (!w || !gravity) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    for (int k = 0; k < 3; k++) { w->cfg.gravity[k] = gravity[k]; w->dw.gravityAcc[k] = gravity[k]; }
    return body_gravity(w, nullptr, gravity, 0, true);
}

int jbgpu_world_set_body_gravity(jbgpu_world* w, const int32_t* bodies, const float* acc, int32_t n) {
    if (!w || n < 0 || (n > 0 && (!bodies || !acc))) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad gravity arguments");
    for (int k = 0; k < n; k++)
        if (bodies[k] < 0 || bodies[k] >= w->nBodies) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad body index");
    return n == 0 ? JBGPU_OK : body_gravity(w, bodies, acc, n, false);
}

int jbgpu_world_get_residual_trace(jbgpu_world* w, float* out, int32_t cap, int32_t* n) {
    if (!w || !n || cap < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad arguments");
    CK(cudaSetDevice(w->device));
    *n = 0;
    if (!(w->dw.resTol > 0.0f) || !w->sb.resTrace) return JBGPU_OK;
    int iters = 0;
    CK(cudaMemcpyAsync(&iters, w->dw.ctr + C_PGS_ITERS, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    iters = std::max(0, std::min(iters, (int)JBGPU_RESIDUAL_TRACE_MAX));
    *n = iters;
    if (!out || iters == 0) return JBGPU_OK;
    if (cap < iters) return fail(JBGPU_ERR_CAPACITY, "caller buffer too small");
    CK(cudaMemcpyAsync(out, w->sb.resTrace, sizeof(float) * 2 * iters, cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    return JBGPU_OK;
}

int jbgpu_world_set_solver_iterations(jbgpu_world* w, int32_t num_iterations, float residual, int32_t max_iterations) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    if (num_iterations < 0 || max_iterations < 0 || !(residual >= 0.0f))
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "negative iteration count or residual");
    CK(cudaSetDevice(w->device));
    CK(cudaStreamSynchronize(w->stream));
    w->cfg.num_iterations = num_iterations;
    w->cfg.solver_residual = residual;
    w->cfg.solver_max_iterations = max_iterations;
    graphs_clear(w);
    w->dw.numIter = num_iterations;
    w->dw.resTol = residual;
    w->dw.maxIter = max_iterations > 0 ? max_iterations : 200;
    return JBGPU_OK;
}

int jbgpu_world_set_warmstart_mlp(jbgpu_world* w, jbgpu_mlp* mlp) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    CK(cudaSetDevice(w->device));
    if (mlp && !w->learnReady) {
        if (solver_learn_configure()) return fail(JBGPU_ERR_CUDA, "warm-start kernel shared-memory size");
        w->learnReady = true;
    }
    CK(cudaStreamSynchronize(w->stream));
    w->mlp = mlp;
    return JBGPU_OK;
}

int jbgpu_world_set_sample_logging(jbgpu_world* w, int32_t on) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    if (on < 0 || on > 2) return fail(JBGPU_ERR_INVALID_ARGUMENT, "sample logging is 0, 1 or 2");
    w->logSamples = on != 0;
    w->logAll = on == 2;
    return JBGPU_OK;
}

int jbgpu_world_get_samples(jbgpu_world* w, float* x, float* t, int32_t capacity, int32_t* n) {
    if (!w || !n) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    *n = 0;
    if (!w->logSamples || !w->sampleX) return JBGPU_OK;
    CK(cudaSetDevice(w->device));
    cudaStream_t s = w->stream;
    int nc = 0, np = 0;
    CK(cudaMemcpyAsync(&nc, w->sb.nCand, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&np, w->rows.nPts, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (nc <= 0 || np <= 0) return JBGPU_OK;
    std::vector<float> X((size_t)np * JBGPU_MLP_INPUTS), T((size_t)np * JBGPU_MLP_OUTPUTS);
    CK(cudaMemcpyAsync(X.data(), w->sampleX, sizeof(float) * X.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(T.data(), w->sampleT, sizeof(float) * T.size(), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int cnt = 0;
    for (int q = 0; q < np; q++) {
        if (std::isnan(T[(size_t)q * JBGPU_MLP_OUTPUTS])) continue;   // island not converged
        if (cnt < capacity && x && t) {
            std::memcpy(x + (size_t)cnt * JBGPU_MLP_INPUTS, &X[(size_t)q * JBGPU_MLP_INPUTS], sizeof(float) * JBGPU_MLP_INPUTS);
            std::memcpy(t + (size_t)cnt * JBGPU_MLP_OUTPUTS, &T[(size_t)q * JBGPU_MLP_OUTPUTS], sizeof(float) * JBGPU_MLP_OUTPUTS);
        }
        cnt++;
    }
    *n = cnt;
    if (cnt > capacity && x && t) return fail(JBGPU_ERR_CAPACITY, "sample buffer too small");
    return JBGPU_OK;
}

int jbgpu_world_add_point2point(jbgpu_world* w, int32_t a, int32_t b, const float pa[3], const float pb[3], int32_t* id) {
    if (!w || !pa || !pb) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (a < 0 || a >= w->nBodies || b < -1 || b >= w->nBodies || a == b)
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint bodies");
    w->jKind.push_back(JOINT_P2P);
    w->jA.push_back(a);
    w->jB.push_back(b);
    w->jPivA.push_back(make_float4(pa[0], pa[1], pa[2], 0.0f));
    w->jPivB.push_back(make_float4(pb[0], pb[1], pb[2], 0.0f));
    w->jSet.push_back(make_float4(0.3f, 1.0f, 0.0f, 0.0f));   // ConstraintSetting defaults
    w->jSet2.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (int r = 0; r < 6; r++) w->jFrame.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (int r = 0; r < D6_SET_F4; r++) w->jD6.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    w->jointsDirty = true;
    if (id) *id = (int32_t)w->jA.size() - 1;
    return JBGPU_OK;
}

int jbgpu_world_set_joint_setting(jbgpu_world* w, int32_t id, float tau, float damping, float clamp) {
    if (!w || id < 0 || id >= (int)w->jA.size()) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint id");
    if (w->jKind[id] != JOINT_P2P) return fail(JBGPU_ERR_INVALID_ARGUMENT, "not a point-to-point joint");
    w->jSet[id] = make_float4(tau, damping, clamp, 0.0f);
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_add_hinge(jbgpu_world* w, int32_t a, int32_t b, const float fa[12], const float fb[12], int32_t* id) {
    if (!w || !fa || !fb) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null argument");
    if (a < 0 || a >= w->nBodies || b < -1 || b >= w->nBodies || a == b)
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint bodies");
    w->jKind.push_back(JOINT_HINGE);
    w->jA.push_back(a);
    w->jB.push_back(b);
    w->jPivA.push_back(make_float4(fa[9], fa[10], fa[11], 0.0f));
    w->jPivB.push_back(make_float4(fb[9], fb[10], fb[11], 0.0f));
    w->jSet.push_back(make_float4(1e30f, -1e30f, 0.9f, 0.3f));   // free: lower > upper; softness, bias
    w->jSet2.push_back(make_float4(1.0f, 0.0f, 0.0f, 0.0f));     // relaxation, motor target, max motor impulse
    for (const float* f : {fa, fb})
        for (int r = 0; r < 3; r++) w->jFrame.push_back(make_float4(f[r * 3], f[r * 3 + 1], f[r * 3 + 2], 0.0f));
    for (int r = 0; r < D6_SET_F4; r++) w->jD6.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    w->jointsDirty = true;
    if (id) *id = (int32_t)w->jA.size() - 1;
    return JBGPU_OK;
}

int jbgpu_world_add_generic6dof(jbgpu_world* w, int32_t a, int32_t b, const float fa[12], const float fb[12],
                                int32_t useLinearReferenceFrameA, int32_t* id) {
    int32_t k = -1;
    int rc = jbgpu_world_add_hinge(w, a, b, fa, fb, &k);
    if (rc) return rc;
    w->jKind[k] = JOINT_6DOF;
    w->jSet[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    w->jSet2[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4* d = &w->jD6[(size_t)k * D6_SET_F4];
    d[0] = make_float4(0.0f, 0.0f, 0.0f, useLinearReferenceFrameA ? 1.0f : 0.0f);   // TranslationalLimitMotor:
    d[1] = make_float4(0.0f, 0.0f, 0.0f, 0.7f);                                      // limits 0 (locked), softness,
    d[2] = make_float4(1.0f, 0.5f, 0.0f, 0.0f);                                      // damping, restitution
    for (int i = 0; i < 3; i++) {                                                     // RotationalLimitMotor defaults
        d[3 + 3 * i] = make_float4(-3.40282347e+38f, 3.40282347e+38f, 0.0f, 0.1f);
        d[4 + 3 * i] = make_float4(300.0f, 1.0f, 0.5f, 0.5f);
        d[5 + 3 * i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (id) *id = k;
    return JBGPU_OK;
}

int jbgpu_world_add_cone_twist(jbgpu_world* w, int32_t a, int32_t b, const float fa[12], const float fb[12], int32_t* id) {
    int32_t k = -1;
    int rc = jbgpu_world_add_hinge(w, a, b, fa, fb, &k);
    if (rc) return rc;
    w->jKind[k] = JOINT_CONE;
    w->jSet[k] = make_float4(1e30f, 1e30f, 1e30f, 0.0f);   // spans 1e30; limitSoftness left unset (0)
    w->jSet2[k] = make_float4(0.3f, 1.0f, 0.0f, 0.0f);     // biasFactor, relaxationFactor
    if (id) *id = k;
    return JBGPU_OK;
}

static int cone_id(jbgpu_world* w, int32_t id) {
    if (!w || id < 0 || id >= (int)w->jA.size()) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint id");
    if ((w->jKind[id] & JK_TYPE) != JOINT_CONE) return fail(JBGPU_ERR_INVALID_ARGUMENT, "not a cone-twist joint");
    return JBGPU_OK;
}

int jbgpu_world_set_cone_twist_limit(jbgpu_world* w, int32_t id, float swing1, float swing2, float twist, float softness,
                                     float bias, float relaxation) {
    int rc = cone_id(w, id);
    if (rc) return rc;
    w->jSet[id] = make_float4(swing1, swing2, twist, softness);
    w->jSet2[id] = make_float4(bias, relaxation, 0.0f, 0.0f);
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_set_cone_twist_angular_only(jbgpu_world* w, int32_t id, int32_t on) {
    int rc = cone_id(w, id);
    if (rc) return rc;
    w->jKind[id] = on ? (w->jKind[id] | JK_ANGULAR_ONLY) : (w->jKind[id] & ~JK_ANGULAR_ONLY);
    w->jointsDirty = true;
    return JBGPU_OK;
}

// SliderConstraint.initParams (SliderConstraint.java:139-172) in jbgpu_world_set_slider_params order.
static const float kSliderDefaults[JBGPU_SLIDER_PARAMS] = {
    1.0f, -1.0f, 0.0f, 0.0f,            // lower / upper linear limit, lower / upper angular limit
    1.0f, 0.7f, 0.0f, 1.0f, 0.7f, 0.0f, // softness, restitution, damping: dir lin, dir ang
    1.0f, 0.7f, 1.0f, 1.0f, 0.7f, 1.0f, // lim lin, lim ang
    1.0f, 0.7f, 1.0f, 1.0f, 0.7f, 1.0f, // ortho lin, ortho ang
    0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f  // linear motor (on, target velocity, max force), angular motor
};

int jbgpu_world_add_slider(jbgpu_world* w, int32_t a, int32_t b, const float fa[12], const float fb[12],
                           int32_t useLinearReferenceFrameA, int32_t* id) {
    int32_t k = -1;
    int rc = jbgpu_world_add_hinge(w, a, b, fa, fb, &k);
    if (rc) return rc;
    w->jKind[k] = JOINT_SLIDER;
    w->jSet[k] = make_float4(useLinearReferenceFrameA ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
    w->jSet2[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    std::memcpy(&w->jD6[(size_t)k * D6_SET_F4], kSliderDefaults, sizeof(kSliderDefaults));
    if (id) *id = k;
    return JBGPU_OK;
}

int jbgpu_world_set_slider_params(jbgpu_world* w, int32_t id, const float* params) {
    if (!w || id < 0 || id >= (int)w->jA.size() || !params) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint id");
    if ((w->jKind[id] & JK_TYPE) != JOINT_SLIDER) return fail(JBGPU_ERR_INVALID_ARGUMENT, "not a slider");
    std::memcpy(&w->jD6[(size_t)id * D6_SET_F4], params, sizeof(float) * JBGPU_SLIDER_PARAMS);
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_get_slider_params(jbgpu_world* w, int32_t id, float* params) {
    if (!w || id < 0 || id >= (int)w->jA.size() || !params) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint id");
    if ((w->jKind[id] & JK_TYPE) != JOINT_SLIDER) return fail(JBGPU_ERR_INVALID_ARGUMENT, "not a slider");
    std::memcpy(params, &w->jD6[(size_t)id * D6_SET_F4], sizeof(float) * JBGPU_SLIDER_PARAMS);
    return JBGPU_OK;
}

static int d6_id(jbgpu_world* w, int32_t id) {
    if (!w || id < 0 || id >= (int)w->jA.size()) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint id");
    if ((w->jKind[id] & JK_TYPE) != JOINT_6DOF) return fail(JBGPU_ERR_INVALID_ARGUMENT, "not a generic 6-dof joint");
    return JBGPU_OK;
}

int jbgpu_world_set_6dof_limit(jbgpu_world* w, int32_t id, int32_t axis, float lo, float hi) {
    int rc = d6_id(w, id);
    if (rc) return rc;
    if (axis < 0 || axis > 5) return fail(JBGPU_ERR_INVALID_ARGUMENT, "axis 0..5");
    float4* d = &w->jD6[(size_t)id * D6_SET_F4];
    if (axis < 3) {
        float* lo3 = &d[0].x;
        float* hi3 = &d[1].x;
        lo3[axis] = lo;
        hi3[axis] = hi;
    } else {
        d[3 + 3 * (axis - 3)].x = lo;
        d[3 + 3 * (axis - 3)].y = hi;
    }
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_set_6dof_linear_motor(jbgpu_world* w, int32_t id, float softness, float damping, float restitution) {
    int rc = d6_id(w, id);
    if (rc) return rc;
    float4* d = &w->jD6[(size_t)id * D6_SET_F4];
    d[1].w = softness;
    d[2].x = damping;
    d[2].y = restitution;
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_set_6dof_angular_motor(jbgpu_world* w, int32_t id, int32_t axis, int32_t enable, float targetVelocity,
                                       float maxMotorForce, float maxLimitForce, float damping, float softness, float erp,
                                       float bounce) {
    int rc = d6_id(w, id);
    if (rc) return rc;
    if (axis < 0 || axis > 2) return fail(JBGPU_ERR_INVALID_ARGUMENT, "angular axis 0..2");
    float4* d = &w->jD6[(size_t)id * D6_SET_F4 + 3 + 3 * axis];
    d[0].z = targetVelocity;
    d[0].w = maxMotorForce;
    d[1] = make_float4(maxLimitForce, damping, softness, erp);
    d[2] = make_float4(bounce, enable ? 1.0f : 0.0f, 0.0f, 0.0f);
    w->jointsDirty = true;
    return JBGPU_OK;
}

static int hinge_id(jbgpu_world* w, int32_t id) {
    if (!w || id < 0 || id >= (int)w->jA.size()) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint id");
    if ((w->jKind[id] & JK_TYPE) != JOINT_HINGE) return fail(JBGPU_ERR_INVALID_ARGUMENT, "not a hinge");
    return JBGPU_OK;
}

int jbgpu_world_set_hinge_limit(jbgpu_world* w, int32_t id, float low, float high, float softness, float bias,
                                float relaxation) {
    int rc = hinge_id(w, id);
    if (rc) return rc;
    w->jSet[id] = make_float4(low, high, softness, bias);
    w->jSet2[id].x = relaxation;
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_enable_hinge_motor(jbgpu_world* w, int32_t id, int32_t enable, float target, float maxImpulse) {
    int rc = hinge_id(w, id);
    if (rc) return rc;
    w->jKind[id] = enable ? (w->jKind[id] | JK_MOTOR) : (w->jKind[id] & ~JK_MOTOR);
    w->jSet2[id].y = target;
    w->jSet2[id].z = maxImpulse;
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_set_hinge_angular_only(jbgpu_world* w, int32_t id, int32_t on) {
    int rc = hinge_id(w, id);
    if (rc) return rc;
    w->jKind[id] = on ? (w->jKind[id] | JK_ANGULAR_ONLY) : (w->jKind[id] & ~JK_ANGULAR_ONLY);
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_remove_joint(jbgpu_world* w, int32_t id) {
    if (!w || id < 0 || id >= (int)w->jA.size()) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad joint id");
    auto drop = [id](auto& v, size_t per) { v.erase(v.begin() + (size_t)id * per, v.begin() + (size_t)(id + 1) * per); };
    drop(w->jKind, 1); drop(w->jA, 1); drop(w->jB, 1); drop(w->jPivA, 1); drop(w->jPivB, 1);
    drop(w->jSet, 1); drop(w->jSet2, 1); drop(w->jFrame, 6); drop(w->jD6, D6_SET_F4);
    DevJoints& J = w->sb.J;
    if (id < J.n) {   // the solved joints' applied impulses move down with them
        CK(cudaSetDevice(w->device));
        std::vector<float> imp(J.n);
        CK(cudaMemcpyAsync(imp.data(), J.imp, sizeof(float) * J.n, cudaMemcpyDeviceToHost, w->stream));
        CK(cudaStreamSynchronize(w->stream));
        imp.erase(imp.begin() + id);
        J.n -= 1;
        if (J.n > 0) {
            CK(cudaMemcpyAsync(J.imp, imp.data(), sizeof(float) * J.n, cudaMemcpyHostToDevice, w->stream));
            CK(cudaStreamSynchronize(w->stream));
        }
    }
    w->jointsDirty = true;
    return JBGPU_OK;
}

int jbgpu_world_get_joint_impulses(jbgpu_world* w, float* out, int32_t cap, int32_t* n) {
    if (!w || !n) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null argument");
    const int nj = (int)w->jA.size();
    *n = nj;
    if (!out || nj == 0) return JBGPU_OK;
    if (nj > cap) return fail(JBGPU_ERR_CAPACITY, "caller buffer too small");
    CK(cudaSetDevice(w->device));
    if (w->sb.J.n < nj) {   // joints added since the last step: not solved yet
        std::fill(out, out + nj, 0.0f);
        if (w->sb.J.n == 0) return JBGPU_OK;
    }
    CK(cudaMemcpyAsync(out, w->sb.J.imp, sizeof(float) * w->sb.J.n, cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    return JBGPU_OK;
}

int jbgpu_world_timer(jbgpu_world* w, int32_t mark, double* ms) {
    if (!w || (mark != 0 && mark != 1) || (mark == 1 && !ms)) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad arguments");
    CK(cudaSetDevice(w->device));
    if (mark == 0) {
        CK(cudaEventRecord(w->evT0, w->stream));
        return JBGPU_OK;
    }
    CK(cudaEventRecord(w->evT1, w->stream));
    CK(cudaEventSynchronize(w->evT1));
    float t = 0.0f;
    CK(cudaEventElapsedTime(&t, w->evT0, w->evT1));
    *ms = t;
    return JBGPU_OK;
}

int jbgpu_world_ray_test(jbgpu_world* w, const float* from, const float* to, const int32_t* rayWorld, int32_t n,
                         int32_t group, int32_t mask, int32_t deviceBuffers, jbgpu_ray_hit* hits) {
    if (!w || n < 0 || (n > 0 && (!from || !to || !hits))) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad ray arguments");
    if (n == 0) return JBGPU_OK;
    CK(cudaSetDevice(w->device));
    int rc = prepare(w);
    if (rc) return rc;
    cudaStream_t s = w->stream;
    if (!deviceBuffers && rayWorld)
        for (int i = 0; i < n; i++)
            if (rayWorld[i] < 0 || rayWorld[i] >= w->nWorlds) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad ray world");
    if (w->nBodies == 0) {
        jbgpu_ray_hit miss;
        std::memset(&miss, 0, sizeof(miss));
        miss.body = -1;
        miss.fraction = 1.0f;
        if (deviceBuffers) {
            std::vector<jbgpu_ray_hit> m(n, miss);
            CK(cudaMemcpyAsync(hits, m.data(), sizeof(jbgpu_ray_hit) * n, cudaMemcpyHostToDevice, s));
            CK(cudaStreamSynchronize(s));
        } else {
            std::fill(hits, hits + n, miss);
        }
        return JBGPU_OK;
    }
    DevWorld d = dev_view(w);
    QueryBuffers& Q = w->qb;
    CK(cudaMemsetAsync(w->dw.ctr + C_STATUS, 0, sizeof(int), s));   // traversal-stack and world-id flags of this call
    rc = query_prepare(d, w->bb, Q, s);
    if (rc) return fail(rc, "ray query preparation failed");
    const float* df = from;
    const float* dt = to;
    const int* dw = rayWorld;
    jbgpu_ray_hit* dh = hits;
    if (!deviceBuffers) {
        if (n > Q.capIo) {
            dfree(Q.from); dfree(Q.to); dfree(Q.rayWorld); dfree(Q.hits);
            const int c = std::max(n, 2 * Q.capIo);
            Q.capIo = 0;
            CK(dalloc(&Q.from, 3 * (size_t)c)); CK(dalloc(&Q.to, 3 * (size_t)c)); CK(dalloc(&Q.rayWorld, c)); CK(dalloc(&Q.hits, c));
            Q.capIo = c;
        }
        CK(cudaMemcpyAsync(Q.from, from, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(Q.to, to, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
        if (rayWorld) CK(cudaMemcpyAsync(Q.rayWorld, rayWorld, sizeof(int) * n, cudaMemcpyHostToDevice, s));
        df = Q.from;
        dt = Q.to;
        dw = rayWorld ? Q.rayWorld : nullptr;
        dh = Q.hits;
    }
    rc = query_rays(d, w->bb, Q, df, dt, dw, n, group, mask, dh, w->sms, s);
    if (rc) return fail(rc, rc == JBGPU_ERR_CAPACITY ? "too many (ray, body) candidates in one batch: split the batch"
                                                     : "ray query failed");
    if (!deviceBuffers) CK(cudaMemcpyAsync(hits, Q.hits, sizeof(jbgpu_ray_hit) * n, cudaMemcpyDeviceToHost, s));
    return check_status(w);   // a traversal stack overflow or a bad world id is an error, not a silent miss
}

int jbgpu_world_convex_sweep_test(jbgpu_world* w, int32_t shape, const float* from, const float* to,
                                  const int32_t* sweepWorld, int32_t n, int32_t group, int32_t mask, int32_t deviceBuffers,
                                  jbgpu_ray_hit* hits) {
    if (!w || n < 0 || (n > 0 && (!from || !to || !hits))) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad sweep arguments");
    if (shape < 0 || shape >= (int)w->shapes.size() || !shape_is_convex(w->shapes[shape].type))
        return fail(JBGPU_ERR_INVALID_ARGUMENT, "the cast shape must be a convex shape of the world");
    if (n == 0) return JBGPU_OK;
    if (!deviceBuffers && sweepWorld)
        for (int i = 0; i < n; i++)
            if (sweepWorld[i] < 0 || sweepWorld[i] >= w->nWorlds) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad sweep world");
    CK(cudaSetDevice(w->device));
    int rc = prepare(w);
    if (rc) return rc;
    cudaStream_t s = w->stream;
    if (w->nBodies == 0) {
        jbgpu_ray_hit miss;
        std::memset(&miss, 0, sizeof(miss));
        miss.body = -1;
        miss.fraction = 1.0f;
        if (deviceBuffers) {
            std::vector<jbgpu_ray_hit> m(n, miss);
            CK(cudaMemcpyAsync(hits, m.data(), sizeof(jbgpu_ray_hit) * n, cudaMemcpyHostToDevice, s));
            CK(cudaStreamSynchronize(s));
        } else {
            std::fill(hits, hits + n, miss);
        }
        return JBGPU_OK;
    }
    DevWorld d = dev_view(w);
    QueryBuffers& Q = w->qb;
    CK(cudaMemsetAsync(w->dw.ctr + C_STATUS, 0, sizeof(int), s));   // traversal-stack and world-id flags of this call
    rc = query_prepare(d, w->bb, Q, s);
    if (rc) return fail(rc, "sweep query preparation failed");
    if (deviceBuffers) {
        rc = query_sweeps(d, w->bb, Q, shape, from, to, sweepWorld, n, group, mask, hits, w->sms, s);
        if (rc) return fail(rc, rc == JBGPU_ERR_CAPACITY ? "too many (sweep, body) candidates in one batch: split the batch"
                                                         : "sweep query failed");
        return check_status(w);
    }
    float *df = nullptr, *dt = nullptr;
    int* dw = nullptr;
    jbgpu_ray_hit* dh = nullptr;
    cudaError_t e = dalloc(&df, 12 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(&dt, 12 * (size_t)n);
    if (e == cudaSuccess && sweepWorld) e = dalloc(&dw, (size_t)n);
    if (e == cudaSuccess) e = dalloc(&dh, (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(df, from, sizeof(float) * 12 * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, to, sizeof(float) * 12 * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && sweepWorld) e = cudaMemcpyAsync(dw, sweepWorld, sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) rc = query_sweeps(d, w->bb, Q, shape, df, dt, dw, n, group, mask, dh, w->sms, s);
    if (e == cudaSuccess && !rc) e = cudaMemcpyAsync(hits, dh, sizeof(jbgpu_ray_hit) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dfree(df); dfree(dt); dfree(dw); dfree(dh);
    if (e != cudaSuccess) return fail(JBGPU_ERR_CUDA, cudaGetErrorString(e));
    if (rc) return fail(rc, rc == JBGPU_ERR_CAPACITY ? "too many (sweep, body) candidates in one batch: split the batch"
                                                     : "sweep query failed");
    return check_status(w);
}

int jbgpu_world_set_graph(jbgpu_world* w, int32_t on) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    CK(cudaSetDevice(w->device));
    CK(cudaStreamSynchronize(w->stream));
    graphs_clear(w);
    w->graphOn = on != 0;
    w->graphError.clear();
    return JBGPU_OK;
}

int jbgpu_world_graph_status(jbgpu_world* w, int32_t* graphs, const char** error) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    if (graphs) *graphs = (int32_t)w->graphs.size();
    if (error) *error = w->graphError.c_str();
    return JBGPU_OK;
}

int jbgpu_world_set_ray_replay(jbgpu_world* w, int32_t all) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    w->qb.replayAll = all != 0;
    return JBGPU_OK;
}

int jbgpu_world_synchronize(jbgpu_world* w) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    CK(cudaStreamSynchronize(w->stream));
    return JBGPU_OK;
}

int jbgpu_world_get_state(jbgpu_world* w, jbgpu_state* st) {
    if (!w || !st) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    CK(cudaSetDevice(w->device));
    int n = w->nBodies;
    st->n_bodies = n;
    if (n == 0) return JBGPU_OK;
    cudaStream_t s = w->stream;
    DevWorld& D = w->dw;
    std::vector<float4> a(n), b(n), c(n);
    auto get4 = [&](float4* src, std::vector<float4>& dst) -> int { CK(cudaMemcpyAsync(dst.data(), src, sizeof(float4) * n, cudaMemcpyDeviceToHost, s)); return 0; };
    int rc;
    if (st->transform) {
        if ((rc = get4(D.xr0, a)) || (rc = get4(D.xr1, b)) || (rc = get4(D.xr2, c))) return rc;
        CK(cudaStreamSynchronize(s));
        for (int i = 0; i < n; i++) {
            float* t = st->transform + 12 * i;
            t[0] = a[i].x; t[1] = a[i].y; t[2] = a[i].z; t[3] = b[i].x; t[4] = b[i].y; t[5] = b[i].z;
            t[6] = c[i].x; t[7] = c[i].y; t[8] = c[i].z; t[9] = a[i].w; t[10] = b[i].w; t[11] = c[i].w;
        }
    }
    if (st->inv_inertia_world) {
        if ((rc = get4(D.iw0, a)) || (rc = get4(D.iw1, b)) || (rc = get4(D.iw2, c))) return rc;
        CK(cudaStreamSynchronize(s));
        for (int i = 0; i < n; i++) {
            float* t = st->inv_inertia_world + 9 * i;
            t[0] = a[i].x; t[1] = a[i].y; t[2] = a[i].z; t[3] = b[i].x; t[4] = b[i].y; t[5] = b[i].z;
            t[6] = c[i].x; t[7] = c[i].y; t[8] = c[i].z;
        }
    }
    auto get3 = [&](float4* src, float* dst) -> int {
        if (!dst) return 0;
        CK(cudaMemcpyAsync(a.data(), src, sizeof(float4) * n, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        for (int i = 0; i < n; i++) { dst[3 * i] = a[i].x; dst[3 * i + 1] = a[i].y; dst[3 * i + 2] = a[i].z; }
        return 0;
    };
    if ((rc = get3(D.linvel, st->linear_velocity)) || (rc = get3(D.angvel, st->angular_velocity)) ||
        (rc = get3(D.force, st->total_force)) || (rc = get3(D.torque, st->total_torque)))
        return rc;
    if (st->aabb) {
        if ((rc = get4(D.amin, a)) || (rc = get4(D.amax, b))) return rc;
        CK(cudaStreamSynchronize(s));
        for (int i = 0; i < n; i++) {
            float* t = st->aabb + 6 * i;
            t[0] = a[i].x; t[1] = a[i].y; t[2] = a[i].z; t[3] = b[i].x; t[4] = b[i].y; t[5] = b[i].z;
        }
    }
    if (st->activation_state) CK(cudaMemcpyAsync(st->activation_state, D.act, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    if (st->deactivation_time) CK(cudaMemcpyAsync(st->deactivation_time, D.deact, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    if (st->island_tag) CK(cudaMemcpyAsync(st->island_tag, D.island, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return JBGPU_OK;
}

int jbgpu_world_set_state(jbgpu_world* w, const jbgpu_state* st) {
    if (!w || !st) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    if (st->n_bodies != w->nBodies) return fail(JBGPU_ERR_INVALID_ARGUMENT, "body count mismatch");
    CK(cudaSetDevice(w->device));
    int n = w->nBodies;
    if (n == 0) return JBGPU_OK;
    cudaStream_t s = w->stream;
    DevWorld& D = w->dw;
    std::vector<float4> a(n), b(n), c(n);
    if (st->transform) {
        for (int i = 0; i < n; i++) {
            const float* t = st->transform + 12 * i;
            a[i] = make_float4(t[0], t[1], t[2], t[9]); b[i] = make_float4(t[3], t[4], t[5], t[10]); c[i] = make_float4(t[6], t[7], t[8], t[11]);
        }
        CK(cudaMemcpyAsync(D.xr0, a.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.xr1, b.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.xr2, c.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
    }
    if (st->inv_inertia_world) {
        for (int i = 0; i < n; i++) {
            const float* t = st->inv_inertia_world + 9 * i;
            a[i] = make_float4(t[0], t[1], t[2], 0); b[i] = make_float4(t[3], t[4], t[5], 0); c[i] = make_float4(t[6], t[7], t[8], 0);
        }
        CK(cudaMemcpyAsync(D.iw0, a.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.iw1, b.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.iw2, c.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
    }
    auto put3 = [&](float4* dst, const float* src) -> int {
        if (!src) return 0;
        for (int i = 0; i < n; i++) a[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], 0);
        CK(cudaMemcpyAsync(dst, a.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
        return 0;
    };
    int rc;
    if ((rc = put3(D.linvel, st->linear_velocity)) || (rc = put3(D.angvel, st->angular_velocity)) ||
        (rc = put3(D.force, st->total_force)) || (rc = put3(D.torque, st->total_torque)))
        return rc;
    if (st->aabb) {
        for (int i = 0; i < n; i++) {
            const float* t = st->aabb + 6 * i;
            a[i] = make_float4(t[0], t[1], t[2], 0); b[i] = make_float4(t[3], t[4], t[5], 0);
        }
        CK(cudaMemcpyAsync(D.amin, a.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(D.amax, b.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    }
    if (st->activation_state) CK(cudaMemcpyAsync(D.act, st->activation_state, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    if (st->deactivation_time) CK(cudaMemcpyAsync(D.deact, st->deactivation_time, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    return JBGPU_OK;
}

int jbgpu_world_get_pairs(jbgpu_world* w, uint64_t* keys, int32_t cap, int32_t* n) {
    if (!w || !n) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    *n = w->nPairs;
    if (w->nPairs > cap) return fail(JBGPU_ERR_CAPACITY, "caller buffer too small");
    if (w->nPairs && keys) {
        CK(cudaMemcpyAsync(keys, w->pairs[w->cur].keys, sizeof(uint64_t) * w->nPairs, cudaMemcpyDeviceToHost, w->stream));
        CK(cudaStreamSynchronize(w->stream));
    }
    return JBGPU_OK;
}

int jbgpu_world_get_manifolds(jbgpu_world* w, jbgpu_manifolds* m) {
    if (!w || !m) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    int np = w->nPairs;
    m->n_pairs = np;
    if (np > m->capacity) return fail(JBGPU_ERR_CAPACITY, "caller buffer too small");
    if (np == 0) return JBGPU_OK;
    cudaStream_t s = w->stream;
    DevPairs& P = w->pairs[w->cur];
    std::vector<int> has(np), cnt(np);
    std::vector<float4> f[8];
    float4* src[8] = {P.pA, P.pB, P.wA, P.wB, P.nrm, P.imp, P.d1, P.d2};
    if (m->keys) CK(cudaMemcpyAsync(m->keys, P.keys, sizeof(uint64_t) * np, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(has.data(), P.has, sizeof(int) * np, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(cnt.data(), P.n, sizeof(int) * np, cudaMemcpyDeviceToHost, s));
    if (m->points)
        for (int k = 0; k < 8; k++) {
            f[k].resize((size_t)np * 4);
            CK(cudaMemcpyAsync(f[k].data(), src[k], sizeof(float4) * np * 4, cudaMemcpyDeviceToHost, s));
        }
    CK(cudaStreamSynchronize(s));
    for (int i = 0; i < np; i++) {
        int nn = has[i] ? cnt[i] : 0;
        if (m->flags) m->flags[i] = has[i] ? 1 : 0;
        if (m->num_points) m->num_points[i] = nn;
        if (!m->points) continue;
        for (int j = 0; j < 4; j++) {
            float* o = m->points + ((size_t)i * 4 + j) * JBGPU_POINT_FLOATS;
            std::memset(o, 0, sizeof(float) * JBGPU_POINT_FLOATS);
            if (j >= nn) continue;
            size_t k = (size_t)i * 4 + j;
            float4 pA = f[0][k], pB = f[1][k], wA = f[2][k], wB = f[3][k], nr = f[4][k], im = f[5][k], d1 = f[6][k], d2 = f[7][k];
            o[0] = pA.x; o[1] = pA.y; o[2] = pA.z; o[3] = pB.x; o[4] = pB.y; o[5] = pB.z;
            o[6] = wA.x; o[7] = wA.y; o[8] = wA.z; o[9] = wB.x; o[10] = wB.y; o[11] = wB.z;
            o[12] = nr.x; o[13] = nr.y; o[14] = nr.z; o[15] = pA.w; o[16] = wA.w; o[17] = wB.w;
            o[18] = nr.w; o[19] = im.x; o[20] = im.y; o[21] = im.z;
            int life;
            std::memcpy(&life, &pB.w, 4);
            o[22] = (float)life;
            o[23] = d1.x; o[24] = d1.y; o[25] = d1.z; o[26] = d2.x; o[27] = d2.y; o[28] = d2.z;
        }
    }
    return JBGPU_OK;
}

int jbgpu_world_set_manifolds(jbgpu_world* w, const jbgpu_manifolds* m) {
    if (!w || !m || m->n_pairs < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    CK(cudaSetDevice(w->device));
    graphs_clear(w);
    int rc = prepare(w);
    if (rc) return rc;
    int np = m->n_pairs;
    if ((rc = ensure_pair_capacity(w, w->cur, std::max(np, 1)))) return rc;
    cudaStream_t s = w->stream;
    DevPairs& P = w->pairs[w->cur];
    std::vector<int> has(np), cnt(np), b0(np), b1(np);
    std::vector<float4> f[8];
    for (int k = 0; k < 8; k++) f[k].assign((size_t)np * 4, make_float4(0, 0, 0, 0));
    for (int i = 0; i < np; i++) {
        uint64_t key = m->keys[i];
        int a = key_owner(key), b = key_partner(key);
        if (a < 0 || b < 0 || a >= w->nBodies || b >= w->nBodies || a == b) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad pair key");
        if (i > 0 && m->keys[i - 1] >= key) return fail(JBGPU_ERR_INVALID_ARGUMENT, "keys not strictly ascending");
        const HostShape& sl = w->shapes[w->hShape[std::min(a, b)]];
        const HostShape& sh = w->shapes[w->hShape[std::max(a, b)]];
        if (key_sub(key) >= std::max(1, sl.child_cnt) * std::max(1, sh.child_cnt))
            return fail(JBGPU_ERR_INVALID_ARGUMENT, "pair key names a child combination the bodies do not have");
        manifold_bodies(a, b, sl.type, sh.type, b0[i], b1[i]);
        has[i] = (m->flags[i] & 1) ? 1 : 0;
        cnt[i] = has[i] ? m->num_points[i] : 0;
        if (cnt[i] < 0 || cnt[i] > 4) return fail(JBGPU_ERR_INVALID_ARGUMENT, "num_points out of range");
        for (int j = 0; j < cnt[i]; j++) {
            const float* o = m->points + ((size_t)i * 4 + j) * JBGPU_POINT_FLOATS;
            size_t k = (size_t)i * 4 + j;
            int life = (int)o[22];
            float lifef;
            std::memcpy(&lifef, &life, 4);
            f[0][k] = make_float4(o[0], o[1], o[2], o[15]);
            f[1][k] = make_float4(o[3], o[4], o[5], lifef);
            f[2][k] = make_float4(o[6], o[7], o[8], o[16]);
            f[3][k] = make_float4(o[9], o[10], o[11], o[17]);
            f[4][k] = make_float4(o[12], o[13], o[14], o[18]);
            f[5][k] = make_float4(o[19], o[20], o[21], 0.0f);
            f[6][k] = make_float4(o[23], o[24], o[25], 0.0f);
            f[7][k] = make_float4(o[26], o[27], o[28], 0.0f);
        }
    }
    if (np) {
        float4* dst[8] = {P.pA, P.pB, P.wA, P.wB, P.nrm, P.imp, P.d1, P.d2};
        CK(cudaMemcpyAsync(P.keys, m->keys, sizeof(uint64_t) * np, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(P.has, has.data(), sizeof(int) * np, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(P.n, cnt.data(), sizeof(int) * np, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(P.b0, b0.data(), sizeof(int) * np, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(P.b1, b1.data(), sizeof(int) * np, cudaMemcpyHostToDevice, s));
        for (int k = 0; k < 8; k++) CK(cudaMemcpyAsync(dst[k], f[k].data(), sizeof(float4) * np * 4, cudaMemcpyHostToDevice, s));
    }
    CK(cudaStreamSynchronize(s));
    w->nPairs = np;
    w->bb.offPrevValid = false;   // the per-owner offsets of the pair array are unknown
    return JBGPU_OK;
}

int jbgpu_world_get_solver_order(jbgpu_world* w, int32_t* out, int32_t cap, int32_t* n) {
    if (!w || !n) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    cudaStream_t s = w->stream;
    int nc = 0, ncol = 0;
    CK(cudaMemcpyAsync(&nc, w->sb.nCand, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&ncol, w->sb.nColours, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *n = nc;
    if (nc > cap) return fail(JBGPU_ERR_CAPACITY, "caller buffer too small");
    if (nc == 0 || !out) return JBGPU_OK;
    std::vector<int> cand(nc), col(nc), bucket(nc);
    CK(cudaMemcpyAsync(cand.data(), w->sb.cand, sizeof(int) * nc, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(col.data(), w->sb.colourOf, sizeof(int) * nc, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(bucket.data(), w->sb.bucket, sizeof(int) * nc, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    // an order equivalent to the solve: by part (cut manifolds last), colour, pair index
    std::vector<std::tuple<int, int, int>> v(nc);
    for (int k = 0; k < nc; k++) v[k] = std::make_tuple(bucket[k], col[k], cand[k]);
    std::sort(v.begin(), v.end());
    for (int k = 0; k < nc; k++) out[k] = std::get<2>(v[k]);
    return JBGPU_OK;
}

int jbgpu_world_counters(jbgpu_world* w, jbgpu_counters* c) {
    if (!w || !c) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    int h[C_NCTR];
    int nc = 0;
    CK(cudaMemcpyAsync(h, w->dw.ctr, sizeof(int) * C_NCTR, cudaMemcpyDeviceToHost, w->stream));
    CK(cudaMemcpyAsync(&nc, w->sb.nCand, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    std::memset(c, 0, sizeof(*c));
    c->steps = w->steps;
    c->bodies = w->nBodies;
    c->pairs = w->nPairs;
    c->manifolds = h[C_MANIFOLDS];
    c->contacts = h[C_CONTACTS];
    c->solver_manifolds = nc;
    c->solver_rows = h[C_ROWS];
    c->colours = h[C_COLOURS];
    c->islands = h[C_ISLANDS];
    c->gjk_calls = h[C_GJK];
    c->epa_calls = h[C_EPA];
    c->status_flags = h[C_STATUS];
    c->solver_iterations = h[C_PGS_ITERS];
    c->cut_colours = h[C_CUT_COLOURS];
    c->cut_manifolds = h[C_CUT_MANIFOLDS];
    c->solver_islands = h[C_ISL_N];
    c->solver_islands_converged = h[C_ISL_CONV];
    c->solver_island_iterations = h[C_ISL_ITERS];
    c->ccd_clamped = w->ccdOn ? h[C_CCD_N] : 0;
    if (w->qb.slowCount) {
        CK(cudaMemcpy(&c->ray_replays, w->qb.slowCount, sizeof(int), cudaMemcpyDeviceToHost));
    }
    return JBGPU_OK;
}

int jbgpu_world_apply_forces(jbgpu_world* w, const float* force, const float* torque) {
    if (!w) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null world");
    if (w->nBodies == 0 || (!force && !torque)) return JBGPU_OK;
    CK(cudaSetDevice(w->device));
    int rc = ensure_io(w);
    if (rc) return rc;
    size_t n3 = (size_t)w->nBodies * 3;
    cudaStream_t s = w->stream;
    if (force) CK(cudaMemcpyAsync(w->ioStage, force, sizeof(float) * n3, cudaMemcpyHostToDevice, s));
    if (torque) CK(cudaMemcpyAsync(w->ioStage + n3, torque, sizeof(float) * n3, cudaMemcpyHostToDevice, s));
    DevWorld d = dev_view(w);
    k_add_forces<<<(w->nBodies + 255) / 256, 256, 0, s>>>(d, force ? w->ioStage : nullptr, torque ? w->ioStage + n3 : nullptr); note_launch();
    CK(cudaGetLastError());
    return JBGPU_OK;
}

int jbgpu_world_get_transforms(jbgpu_world* w, float* out) {
    if (!w || !out) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    if (w->nBodies == 0) return JBGPU_OK;
    CK(cudaSetDevice(w->device));
    int rc = ensure_io(w);
    if (rc) return rc;
    cudaStream_t s = w->stream;
    DevWorld d = dev_view(w);
    k_pack_transforms<<<(w->nBodies + 255) / 256, 256, 0, s>>>(d, w->ioStage); note_launch();
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, w->ioStage, sizeof(float) * 12 * (size_t)w->nBodies, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return JBGPU_OK;
}

int jbgpu_world_get_interpolated_transforms(jbgpu_world* w, float* out) {
    if (!w || !out) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    if (w->nBodies == 0) return JBGPU_OK;
    CK(cudaSetDevice(w->device));
    int rc = ensure_io(w);
    if (rc) return rc;
    cudaStream_t s = w->stream;
    k_pack_interpolated<<<(w->nBodies + 255) / 256, 256, 0, s>>>(dev_view(w), w->localTime, w->ioStage); note_launch();
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, w->ioStage, sizeof(float) * 12 * (size_t)w->nBodies, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return JBGPU_OK;
}

int jbgpu_world_set_profiling(jbgpu_world* w, int32_t max_steps) {
    if (!w || max_steps < 0) return fail(JBGPU_ERR_INVALID_ARGUMENT, "bad arguments");
    CK(cudaSetDevice(w->device));
    CK(cudaStreamSynchronize(w->stream));
    free_prof(w->prof);
    if (w->profHist) cudaFree(w->profHist);
    w->profHist = nullptr;
    if (max_steps == 0) return JBGPU_OK;
    CK(cudaMalloc(&w->profHist, sizeof(int) * (C_NCTR + 1) * (size_t)max_steps));
    size_t ne = (size_t)max_steps * NUM_PHASES * 2;
    w->prof.ev = new cudaEvent_t[ne];
    for (size_t i = 0; i < ne; i++) CK(cudaEventCreate(&w->prof.ev[i]));
    w->prof.maxSteps = max_steps;
    w->prof.step = 0;
    return JBGPU_OK;
}

int jbgpu_world_phase_times(jbgpu_world* w, double* ms, int32_t nph, int32_t* steps) {
    if (!w || !ms) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    CK(cudaStreamSynchronize(w->stream));
    for (int p = 0; p < nph; p++) ms[p] = 0.0;
    const Prof& P = w->prof;
    for (int st = 0; st < P.step; st++)
        for (int p = 0; p < NUM_PHASES && p < nph; p++) {
            float t = 0.0f;
            size_t k = ((size_t)st * NUM_PHASES + p) * 2;
            if (cudaEventElapsedTime(&t, P.ev[k], P.ev[k + 1]) == cudaSuccess) ms[p] += t;
            else cudaGetLastError();
        }
    if (steps) *steps = P.step;
    if (nph > NUM_PHASES && P.step > 0) {   // whole profiled window: first gravity mark to last activation mark
        float t = 0.0f;
        size_t a = (size_t)PH_OTHER * 2, b = (((size_t)(P.step - 1)) * NUM_PHASES + PH_ACTIVATION) * 2 + 1;
        if (cudaEventElapsedTime(&t, P.ev[a], P.ev[b]) == cudaSuccess) ms[NUM_PHASES] = t;
        else cudaGetLastError();
    }
    return JBGPU_OK;
}

int jbgpu_world_profile_counters(jbgpu_world* w, jbgpu_counters* out, int32_t cap, int32_t* n) {
    if (!w || !n) return fail(JBGPU_ERR_INVALID_ARGUMENT, "null");
    int steps = w->prof.step;
    *n = steps;
    if (!out || steps == 0) return JBGPU_OK;
    if (steps > cap) return fail(JBGPU_ERR_CAPACITY, "caller buffer too small");
    std::vector<int> h((size_t)steps * (C_NCTR + 1));
    CK(cudaMemcpyAsync(h.data(), w->profHist, sizeof(int) * h.size(), cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    for (int s = 0; s < steps; s++) {
        const int* c = h.data() + (size_t)s * (C_NCTR + 1);
        jbgpu_counters& o = out[s];
        std::memset(&o, 0, sizeof(o));
        o.bodies = w->nBodies;
        o.pairs = c[C_PAIRS];
        o.manifolds = c[C_MANIFOLDS];
        o.contacts = c[C_CONTACTS];
        o.solver_manifolds = c[C_NCTR];
        o.solver_rows = c[C_ROWS];
        o.colours = c[C_COLOURS];
        o.islands = c[C_ISLANDS];
        o.gjk_calls = c[C_GJK];
        o.epa_calls = c[C_EPA];
        o.status_flags = c[C_STATUS];
        o.solver_iterations = c[C_PGS_ITERS];
        o.cut_colours = c[C_CUT_COLOURS];
        o.cut_manifolds = c[C_CUT_MANIFOLDS];
        o.solver_islands = c[C_ISL_N];
        o.solver_islands_converged = c[C_ISL_CONV];
        o.solver_island_iterations = c[C_ISL_ITERS];
        o.ccd_clamped = c[C_CCD_N];
    }
    return JBGPU_OK;
}

}  // extern "C"

__global__ void k_add_forces(DevWorld w, const float* f, const float* t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    if (f) {   // applyCentralForce: totalForce += force * linearFactor (linearFactor is (1,1,1))
        float4 a = w.force[i];
        w.force[i] = make_float4(__fadd_rn(a.x, f[3 * i]), __fadd_rn(a.y, f[3 * i + 1]), __fadd_rn(a.z, f[3 * i + 2]), 0.0f);
    }
    if (t) {   // applyTorque: totalTorque += torque
        float4 a = w.torque[i];
        w.torque[i] = make_float4(__fadd_rn(a.x, t[3 * i]), __fadd_rn(a.y, t[3 * i + 1]), __fadd_rn(a.z, t[3 * i + 2]), 0.0f);
    }
}

__global__ void k_pack_transforms(DevWorld w, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    float4 a = w.xr0[i], b = w.xr1[i], c = w.xr2[i];
    float* o = out + 12 * (size_t)i;
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = b.x; o[4] = b.y; o[5] = b.z;
    o[6] = c.x; o[7] = c.y; o[8] = c.z; o[9] = a.w; o[10] = b.w; o[11] = c.w;
}

// synchronizeMotionStates (DiscreteDynamicsWorld.java:251-276): a dynamic body's interpolation
// transform integrated by its interpolation velocities over localTime * hitFraction; static and
// kinematic bodies, which the reference leaves out, get their world transform.
__global__ void k_pack_interpolated(DevWorld w, float t, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    jbd::Xf x;
    if (is_static_or_kin(w.flags[i])) {
        x = load_xf(w, i);
    } else {
        const float4 a = w.kx0[i], b = w.kx1[i], c = w.kx2[i];
        jbd::Xf k;
        k.b.r[0] = jbd::mk(a.x, a.y, a.z);
        k.b.r[1] = jbd::mk(b.x, b.y, b.z);
        k.b.r[2] = jbd::mk(c.x, c.y, c.z);
        k.o = jbd::mk(a.w, b.w, c.w);
        x = jbd::integrate_transform(k, jbd::mk4(w.ilv[i]), jbd::mk4(w.iav[i]), __fmul_rn(t, w.hitf[i]));
    }
    float* o = out + 12 * (size_t)i;
    o[0] = x.b.r[0].x; o[1] = x.b.r[0].y; o[2] = x.b.r[0].z; o[3] = x.b.r[1].x; o[4] = x.b.r[1].y; o[5] = x.b.r[1].z;
    o[6] = x.b.r[2].x; o[7] = x.b.r[2].y; o[8] = x.b.r[2].z; o[9] = x.o.x; o[10] = x.o.y; o[11] = x.o.z;
}

// updateInertiaTensor and the creation-time proxy aabb for new bodies.
#include "shapes.cuh"
__global__ void k_init_bodies(DevWorld w, int first, int count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int i = first + k;
    using namespace jbd;
    Xf t = load_xf(w, i);
    M m1 = scaleM(t.b, mk4(w.iloc[i]));
    M iw = mulMM(m1, transpose(t.b));
    w.iw0[i] = f4(iw.r[0], 0.0f);
    w.iw1[i] = f4(iw.r[1], 0.0f);
    w.iw2[i] = f4(iw.r[2], 0.0f);
    V mn, mx;
    shape_aabb(w.sh, w.shape[i], t, mn, mx);
    w.amin[i] = f4(mn, 0.0f);
    w.amax[i] = f4(mx, 0.0f);
    w.island[i] = -1;
}

// CollisionWorld.updateSingleAabb (CollisionWorld.java:195-224): the shape's aabb at the body's
// transform widened by the contact breaking threshold; an oversized box of a non-static body
// disables its simulation.
__global__ void k_shape_aabbs(DevWorld w, int shape) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies || w.shape[i] != shape) return;
    using namespace jbd;
    V mn, mx;
    shape_aabb(w.sh, shape, load_xf(w, i), mn, mx);
    const float c = w.cbt;
    mn = sub(mn, mk(c, c, c));
    mx = add(mx, mk(c, c, c));
    const V d = sub(mx, mn);
    if ((w.flags[i] & CF_STATIC) || (len2(d) < 1e12f)) {
        w.amin[i] = f4(mn, 0.0f);
        w.amax[i] = f4(mx, 0.0f);
    } else {
        w.act[i] = set_activation(w.act[i], DISABLE_SIMULATION);
    }
}
