// Narrowphase: CollisionDispatcher.dispatchAllCollisionPairs for every overlapping pair
// (collision/dispatch/CollisionDispatcher.java:252-257, DefaultNearCallback.java:39-66).
//
// Pass 1 (one thread per pair): needsCollision, algorithm creation (the pair's manifold),
// then sphere-sphere (SphereSphereCollisionAlgorithm.java:73-134), convex-plane
// (ConvexPlaneCollisionAlgorithm.java:75-136) or convex-convex GJK
// (ConvexConvexAlgorithm.java:90-139), adding at most one point and refreshing the
// manifold.  Convex pairs whose GJK ends in the penetration case are queued with their
// partial GJK result.
// Pass 2 (one warp per queued pair, warp-stride over a fixed set of scratch slots, one slot per
// warp): GJK-EPA penetration depth, the deeper-result choice of GjkPairDetector.java:260-303,
// then the same manifold update (lane 0).
#include <mutex>

#include "epa.cuh"
#include "dispatch.cuh"
#include "prims.cuh"
#include "manifold.cuh"
#include "narrowphase.cuh"

namespace jbg {
using namespace jbd;

struct EpaRec {
    int pair;
    int valid;
    float distance;
    float pad;
    float4 pA, pB, nB;
};

JBD void manifold_refresh(Mf& m, const DevWorld& w, int mb0, int mb1) {
    if (m.n == 0) return;
    refresh_points(m, load_xf(w, mb0), load_xf(w, mb1), w.cbt);
}

// Pairs grouped by algorithm before the pass, so that the threads of a warp run the same code:
// bucket 0 = nothing to do (both bodies inactive, or two planes), 1 convex-plane, 2 sphere-
// sphere, then GJK pairs by shape kinds: 3 box-box, 4 with a sphere, 5 with a capsule, 6 with a
// hull, each split by whether the pair's manifold held points after the last step (7-10: the
// same kinds, touching) - separated pairs mostly leave GJK after a few iterations, touching
// ones converge on the contact, so a warp of either kind runs similar iteration counts.  perm
// lists buckets 1..10 in order; the pass covers nPairs - count[0] entries.
JBD int narrow_bucket(const DevWorld& w, const DevPairs& P, int p) {
    uint64_t key = P.keys[p];
    int a = key_owner(key), b = key_partner(key);
    int col0 = min(a, b), col1 = max(a, b);
    if (!is_active_state(w.act[col0]) && !is_active_state(w.act[col1])) return 0;
    int t0, t1;
    const int kind = pair_leaf_types(w, key, col0, col1, t0, t1);
    if (kind == ALG_EMPTY || kind >= ALG_CONVEX_CONCAVE) return 0;   // meshes: the concave pass
    if (kind == ALG_CONVEX_PLANE || kind == ALG_PLANE_CONVEX) return 1;
    if (kind == ALG_SPHERE_SPHERE) return 2;
    const int touching = P.has[p] && P.n[p] > 0 ? 4 : 0;
    if (t0 == SHAPE_HULL || t1 == SHAPE_HULL) return 6 + touching;
    if (t0 == SHAPE_CAPSULE || t1 == SHAPE_CAPSULE) return 5 + touching;
    if (t0 == SHAPE_SPHERE || t1 == SHAPE_SPHERE) return 4 + touching;
    return 3 + touching;
}

// Stable grouping: per block and bucket counts, laid out bucket-major with bucket 0 last, then
// one exclusive scan gives every block its place in every bucket; within a block the pairs
// keep their order (the owner-sorted order of the pair keys, which keeps shape data of an
// owner body in cache).
constexpr int NB_THREADS = 256;
JBD int bucket_row(int v) { return v == 0 ? NB_BUCKETS - 1 : v - 1; }

// Per-warp bucket counts of the block in shared memory (one ballot per bucket, one barrier);
// then a thread's rank among the block's threads of its bucket and each bucket's block count.
JBD void block_bucket_counts(int v, int (*shc)[NB_THREADS / 32]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int u = 0; u < NB_BUCKETS; u++) {
        unsigned m = __ballot_sync(0xffffffffu, v == u);
        if (lane == 0) shc[u][warp] = __popc(m);
    }
    __syncthreads();
}
__global__ void k_narrow_count(DevWorld w, DevPairs P, int nPairs, const int* cntp, unsigned char* bucket, int* blockCnt) {
    __shared__ int shc[NB_BUCKETS][NB_THREADS / 32];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int v = -1;
    if (p < (cntp ? min(nPairs, *cntp) : nPairs)) {
        v = narrow_bucket(w, P, p);
        bucket[p] = (unsigned char)v;
    }
    block_bucket_counts(v, shc);
    if (threadIdx.x < NB_BUCKETS) {
        int total = 0;
        for (int k = 0; k < NB_THREADS / 32; k++) total += shc[threadIdx.x][k];
        blockCnt[bucket_row(threadIdx.x) * gridDim.x + blockIdx.x] = total;
    }
}

__global__ void k_narrow_scatter(int nPairs, const int* cntp, const unsigned char* bucket, const int* blockOff, int* perm) {
    __shared__ int shc[NB_BUCKETS][NB_THREADS / 32];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int v = p < (cntp ? min(nPairs, *cntp) : nPairs) ? bucket[p] : -1;
    block_bucket_counts(v, shc);
    if (v < 0) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int before = 0;
    for (int k = 0; k < warp; k++) before += shc[v][k];
    unsigned mv = 0;
    for (int u = 0; u < NB_BUCKETS; u++) {
        unsigned m = __ballot_sync(__activemask(), v == u);
        if (v == u) mv = m;
    }
    perm[blockOff[bucket_row(v) * gridDim.x + blockIdx.x] + before + __popc(mv & ((1u << lane) - 1u))] = p;
}

// Entries of the pass: the pairs of buckets 1..6 = the start of bucket 0's row.
JBD int narrow_active(const int* blockOff, int nBlocks) { return blockOff[(NB_BUCKETS - 1) * nBlocks]; }

// With perm: n = the grouping's pair blocks and entry i is pair perm[i]; without: n = pairs.
__global__ void __launch_bounds__(128, 4) k_narrow(DevWorld w, DevPairs P, int n, const int* perm, const int* blockOff, EpaRec* queue,
                         int* queueCount, const int* cntp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (perm ? narrow_active(blockOff, n) : (cntp ? min(n, *cntp) : n))) return;
    int p = perm ? perm[i] : i;
    uint64_t key = P.keys[p];
    int a = key_owner(key), b = key_partner(key);
    int col0 = min(a, b), col1 = max(a, b);
    if (!is_active_state(w.act[col0]) && !is_active_state(w.act[col1])) return;   // needsCollision
    Xf x0 = load_xf(w, col0), x1 = load_xf(w, col1);   // the ManifoldResult's root transforms
    Leaf f, g;
    const int kind = pair_leaves(w, key, col0, col1, x0, x1, f, g);
    if (kind == ALG_EMPTY || kind >= ALG_CONVEX_CONCAVE) return;   // no manifold; meshes: the concave pass
    const bool fresh = !P.has[p];            // the algorithm and its manifold come with the first dispatch
    if (fresh) P.has[p] = 1;
    // The collision first, without the manifold (it reads nothing of it), so that GJK's state and
    // the manifold's 4 points are never live together: at most one point for the manifold.
    bool hit = false;
    V nB, pW;
    float dist = 0.0f;
    if (kind == ALG_SPHERE_SPHERE) {
        V diff = sub(f.x.o, g.x.o);
        float l = len(diff);
        float r0 = w.sh.margin[f.shape], r1 = w.sh.margin[g.shape];
        float rs = __fadd_rn(r0, r1);
        if (!(l > rs)) {
            dist = __fsub_rn(l, rs);
            nB = mk(1.0f, 0.0f, 0.0f);
            if (l > FLT_EPS) nB = scl(diff, jdiv(1.0f, l));
            pW = add(g.x.o, scl(nB, r1));
            hit = true;
        }
    } else if (kind == ALG_CONVEX_PLANE || kind == ALG_PLANE_CONVEX) {
        const Leaf& c = kind == ALG_CONVEX_PLANE ? f : g;   // the convex object
        const Leaf& pl = kind == ALG_CONVEX_PLANE ? g : f;
        Xf cx = c.x, px = pl.x;
        ShapeRef cs = shape_ref(w.sh, c.shape);
        float4 plq = w.sh.plane[pl.shape];
        V pn = mk(plq.x, plq.y, plq.z);
        Xf planeInConvex = xf_mul(xf_inverse(cx), px);
        Xf convexInPlane = xf_mul(xf_inverse(px), cx);
        V dir = mulMv(scl(pn, -1.0f), planeInConvex.b);
        V vtx = support_with_margin(cs, dir);
        V vtxInPlane = xf_apply(convexInPlane, vtx);
        float distance = __fsub_rn(dot(pn, vtxInPlane), plq.w);
        V proj = sub(vtxInPlane, scl(pn, distance));
        if (distance < w.cbt) {
            pW = xf_apply(px, proj);
            nB = mulMv(pn, px.b);
            dist = distance;
            hit = true;
        }
    } else {
        ShapeRef sa = shape_ref(w.sh, f.shape), sb = shape_ref(w.sh, g.shape);
        float md = __fadd_rn(__fadd_rn(sa.margin, sb.margin), w.cbt);
        md = __fmul_rn(md, md);
        {   // one counter atomic per group of converged lanes
            const unsigned am = __activemask();
            if ((threadIdx.x & 31) == __ffs(am) - 1) atomicAdd(&w.ctr[C_GJK], __popc(am));
        }
        GjkPart gp = gjk_part(sa, f.x, sb, g.x, md);
        if (gp.needEpa) {
            int q = atomicAdd(queueCount, 1);
            EpaRec r;
            r.pair = p;
            r.valid = gp.isValid ? 1 : 0;
            r.distance = gp.distance;
            r.pad = 0.0f;
            r.pA = f4(gp.pointOnA, 0.0f);
            r.pB = f4(gp.pointOnB, 0.0f);
            r.nB = f4(gp.normalInB, 0.0f);
            queue[q] = r;
            if (fresh) P.n[p] = 0;
            return;   // the EPA pass finishes this pair
        }
        if (gp.isValid) {
            nB = gp.normalInB;
            pW = add(gp.pointOnB, gp.offset);
            dist = gp.distance;
            hit = true;
        }
    }
    // ManifoldResult.addContactPoint and refreshContactPoints on the pair's manifold
    Mf m;
    if (fresh) m.n = 0;
    else load_mf(P, p, m);
    const int mb0 = P.b0[p], mb1 = P.b1[p];
    if (hit)
        add_contact(m, mb0, col0, x0, x1, w.friction[col0], w.friction[col1], w.restitution[col0], w.restitution[col1],
                    nB, pW, dist, w.cbt);
    manifold_refresh(m, w, mb0, mb1);
    store_mf(P, p, m);
}

// One queued pair, by the 32 lanes of a warp (see epa.cuh); lane 0 updates the manifold.  With
// ovfQueue (a reduced-capacity tier) a query that outgrows its slot leaves no result and is queued
// for the tier with the full capacities: EPA is deterministic, so its result does not depend on
// which tier finishes it.  With cand (the concave pass) a queued entry is a (pair, triangle)
// candidate: the convex object against the mesh triangle, the result into res.
__device__ void epa_query(const DevWorld& w, DevPairs& P, const EpaRec* queue, int qi, const EpaSlot& sl, int lane,
                          int* ovfQueue = nullptr, int* ovfCount = nullptr, const int2* cand = nullptr,
                          float4* res = nullptr) {
    EpaRec r = queue[qi];
    const int p = cand ? cand[r.pair].x : r.pair;
    uint64_t key = P.keys[p];
    int a = key_owner(key), b = key_partner(key);
    int col0 = min(a, b), col1 = max(a, b);
    int mb0 = P.b0[p], mb1 = P.b1[p];
    Xf x0 = load_xf(w, col0), x1 = load_xf(w, col1);
    Leaf f, g;
    const int kind = pair_leaves(w, key, col0, col1, x0, x1, f, g);
    ShapeRef sa, sb;
    Xf lA, lB;
    if (cand) {                               // (convex, triangle of the mesh)
        const Leaf& c = kind == ALG_CONVEX_CONCAVE ? f : g;
        const Leaf& t = kind == ALG_CONVEX_CONCAVE ? g : f;
        sa = shape_ref(w.sh, c.shape);
        sb = triangle_ref(w.sh, t.shape, cand[r.pair].y);
        lA = c.x;
        lB = t.x;
    } else {
        sa = shape_ref(w.sh, f.shape);
        sb = shape_ref(w.sh, g.shape);
        lA = f.x;
        lB = g.x;
    }
    V offset = scl(add(lA.o, lB.o), 0.5f);
    lA.o = sub(lA.o, offset);
    lB.o = sub(lB.o, offset);
    bool isValid = r.valid != 0;
    float distance = r.distance;
    V pointOnB = mk4(r.pB), normalInB = mk4(r.nB);
    V wA, wB;
    bool ovf = false;
    if (epa_pen_depth(sa, lA, sb, lB, sl, wA, wB, ovf, lane, 32)) {
        V tn = sub(wB, wA);
        float lenSqr = len2(tn);
        if (lenSqr > __fmul_rn(FLT_EPS, FLT_EPS)) {
            tn = scl(tn, jdiv(1.0f, jsqrt(lenSqr)));
            float distance2 = -len(sub(wA, wB));
            if (!isValid || (distance2 < distance)) {
                distance = distance2;
                pointOnB = wB;
                normalInB = tn;
                isValid = true;
            }
        }
    }
    if (ovf && ovfQueue) {
        if (lane == 0) ovfQueue[atomicAdd(ovfCount, 1)] = qi;
        __syncwarp();
        return;
    }
    if (lane == 0) {
        atomicAdd(&w.ctr[C_EPA], 1);
        if (ovf) atomicOr(&w.ctr[C_STATUS], ST_EPA_POOL);
        if (cand) {
            res[2 * r.pair] = f4(add(pointOnB, offset), distance);
            res[2 * r.pair + 1] = f4(normalInB, isValid ? 1.0f : 0.0f);
        } else {
            Mf m;
            load_mf(P, p, m);
            if (isValid)
                add_contact(m, mb0, col0, x0, x1, w.friction[col0], w.friction[col1], w.restitution[col0],
                            w.restitution[col1], normalInB, add(pointOnB, offset), distance, w.cbt);
            manifold_refresh(m, w, mb0, mb1);
            store_mf(P, p, m);
        }
    }
    __syncwarp();
}

// EPA pass with each warp's polytope in a slot of a global arena.
__global__ void k_narrow_epa(DevWorld w, DevPairs P, const EpaRec* queue, const int* queueCount, EpaArena arena) {
    int n = *queueCount;
    int slot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (slot >= arena.slots) return;
    EpaSlot sl = epa_slot(arena, slot);
    for (int qi = slot; qi < n; qi += arena.slots) epa_query(w, P, queue, qi, sl, lane);
}

// EPA pass with the polytope in shared memory: one warp per block, 97,408 bytes of dynamic
// shared memory (two blocks per SM), blocks stride over the queue.
constexpr size_t EPA_SMEM_BYTES = (size_t)EPA_FACE_CAP * (4 * sizeof(float4) + sizeof(float)) +
                                  (size_t)EPA_MKV_CAP * 2 * sizeof(float4) + (size_t)EPA_SEEN_CAP * sizeof(float4) +
                                  (size_t)EPA_STACK_CAP * sizeof(int2);

// Reduced-capacity tiers: WARPS warps per block, each with a polytope of the given
// capacities in shared memory, taking the queue (list == null) or the previous tier's overflow
// list; queries that outgrow the slot go to this tier's overflow list.  Tier 1 (96 faces, 8
// warps a block) finishes most queries at twice the warps per SM of tier 2 (192 faces, 4 warps).
template <int FACES, int MKV, int SEEN, int STACK>
struct EpaTier {
    static constexpr size_t SLOT_BYTES = (size_t)FACES * (4 * sizeof(float4) + sizeof(float)) +
                                         (size_t)MKV * 2 * sizeof(float4) + (size_t)SEEN * sizeof(float4) +
                                         (size_t)STACK * sizeof(int2);
};
constexpr int EPA_T1_WARPS = 6, EPA_T2_WARPS = 4;
constexpr int EPA_T1_SKIP_STEPS = 8;
using EpaT1 = EpaTier<128, 64, 48, 256>;
using EpaT2 = EpaTier<192, 96, 64, 384>;
constexpr size_t EPA_T1_SMEM_BYTES = EPA_T1_WARPS * EpaT1::SLOT_BYTES;
constexpr size_t EPA_T2_SMEM_BYTES = EPA_T2_WARPS * EpaT2::SLOT_BYTES;

// Tier 1 runs only for a queue longer than tier 2's warps (else its extra warps buy nothing and
// its overflow would be solved twice on the critical path) and while mode (device) is 0; k > 0
// skips it for k more steps, set after a step in which it left more than a third of its queue
// to tier 2.  When tier 1 is skipped, tier 2 takes the queue.
template <int WARPS, int FACES, int MKV, int SEEN, int STACK>
__global__ void __launch_bounds__(32 * WARPS) k_narrow_epa_tier(DevWorld w, DevPairs P, const EpaRec* queue,
                                                                const int* list, const int* count, int* ovfQueue,
                                                                int* ovfCount, const int* mode, const int* queueCount,
                                                                int tier2Warps, const int2* cand, float4* res) {
    extern __shared__ float4 epaSmem[];
    const bool skipped = *mode != 0 || *queueCount <= tier2Warps;   // tier 1 is skipped this step
    if (!list && skipped) return;           // this is tier 1
    if (list && skipped) { list = nullptr; count = queueCount; }   // tier 2 takes the queue
    const int n = *count;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    EpaSlot sl;
    sl.fN = (float4*)((unsigned char*)epaSmem + warp * EpaTier<FACES, MKV, SEEN, STACK>::SLOT_BYTES);
    sl.fV = (int4*)(sl.fN + FACES);
    sl.fF = sl.fV + FACES;
    sl.fE = sl.fF + FACES;
    sl.mW = (float4*)(sl.fE + FACES);
    sl.mR = sl.mW + MKV;
    sl.seen = sl.mR + MKV;
    sl.stack = (int2*)(sl.seen + SEEN);
    sl.fD = (float*)(sl.stack + STACK);
    sl.faceCap = FACES;
    sl.mkvCap = MKV;
    sl.seenCap = SEEN;
    sl.stackCap = STACK;
    const int gw = blockIdx.x * WARPS + warp, nw = gridDim.x * WARPS;
    for (int j = gw; j < n; j += nw) epa_query(w, P, queue, list ? list[j] : j, sl, lane, ovfQueue, ovfCount, cand, res);
}
#define EPA_T1_KERNEL k_narrow_epa_tier<EPA_T1_WARPS, 128, 64, 48, 256>
#define EPA_T2_KERNEL k_narrow_epa_tier<EPA_T2_WARPS, 192, 96, 64, 384>


// Full-capacity tier over the queries the 192-face tier could not finish.
// c: the tier counters (c[0] counts list); block 0 also sets the tier mode of the next step.
__global__ void __launch_bounds__(32) k_narrow_epa_smem(DevWorld w, DevPairs P, const EpaRec* queue, const int* list,
                                                       int* c, const int* queueCount, int tier2Warps,
                                                       const int2* cand, float4* res) {
    extern __shared__ float4 epaSmem[];
    int n = c[0];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int q = *queueCount, m = c[2];
        c[2] = m > 0 ? m - 1 : ((q > tier2Warps && 3 * c[1] > q) ? EPA_T1_SKIP_STEPS : 0);
    }
    EpaSlot sl;
    sl.fN = epaSmem;
    sl.fV = (int4*)(sl.fN + EPA_FACE_CAP);
    sl.fF = sl.fV + EPA_FACE_CAP;
    sl.fE = sl.fF + EPA_FACE_CAP;
    sl.mW = (float4*)(sl.fE + EPA_FACE_CAP);
    sl.mR = sl.mW + EPA_MKV_CAP;
    sl.seen = sl.mR + EPA_MKV_CAP;
    sl.stack = (int2*)(sl.seen + EPA_SEEN_CAP);
    sl.fD = (float*)(sl.stack + EPA_STACK_CAP);
    sl.faceCap = EPA_FACE_CAP;
    sl.mkvCap = EPA_MKV_CAP;
    sl.seenCap = EPA_SEEN_CAP;
    sl.stackCap = EPA_STACK_CAP;
    for (int j = blockIdx.x; j < n; j += gridDim.x) epa_query(w, P, queue, list[j], sl, threadIdx.x, nullptr, nullptr, cand, res);
}

static int gridn_nb(int nPairs) { return (nPairs + NB_THREADS - 1) / NB_THREADS; }

// The three EPA tiers over a queue (queueCount on the device); ovfCount: 3 ints (the two
// overflow lists' counts and the tier mode the last tier sets for the next step).
static void epa_tiers(const DevWorld& w, DevPairs& P, void* queue, int* queueCount, int* ovfQueue, int* ovfQueue2,
                      int* ovfCount, int slots, const int2* cand, float4* res, cudaStream_t s) {
    cudaMemsetAsync(ovfCount, 0, sizeof(int) * 2, s);
    EPA_T1_KERNEL<<<slots, 32 * EPA_T1_WARPS, EPA_T1_SMEM_BYTES, s>>>(
        w, P, (const EpaRec*)queue, nullptr, queueCount, ovfQueue2, ovfCount + 1, ovfCount + 2, queueCount,
        slots * EPA_T2_WARPS, cand, res);
    note_launch();
    EPA_T2_KERNEL<<<slots, 32 * EPA_T2_WARPS, EPA_T2_SMEM_BYTES, s>>>(
        w, P, (const EpaRec*)queue, ovfQueue2, ovfCount + 1, ovfQueue, ovfCount, ovfCount + 2, queueCount,
        slots * EPA_T2_WARPS, cand, res);
    note_launch();
    k_narrow_epa_smem<<<slots, 32, EPA_SMEM_BYTES, s>>>(w, P, (const EpaRec*)queue, ovfQueue, ovfCount, queueCount,
                                                        slots * EPA_T2_WARPS, cand, res);
    note_launch();
}

// Groups the pairs by bucket into nb.perm (blockOff: scanned per-block bucket counts).
static void narrow_group(const DevWorld& w, DevPairs& P, int nPairs, NarrowBuffers& nb, cudaStream_t s,
                         const int* cntp = nullptr) {
    const int blocks = gridn_nb(nPairs);
    k_narrow_count<<<blocks, NB_THREADS, 0, s>>>(w, P, nPairs, cntp, nb.pairBucket, nb.blockOff); note_launch();
    exclusive_scan(nb.blockOff, nb.blockOff, nullptr, NB_BUCKETS * blocks, nb.scanScratch, s);
    k_narrow_scatter<<<blocks, NB_THREADS, 0, s>>>(nPairs, cntp, nb.pairBucket, nb.blockOff, nb.perm); note_launch();
}

void narrowphase_launch(const DevWorld& w, DevPairs& P, int nPairs, NarrowBuffers& nb, cudaStream_t s,
                        const Prof* prof, const int* cntp) {
    if (prof) prof->mark(PH_NARROW, 0, s);
    cudaMemsetAsync(nb.queueCount, 0, sizeof(int), s);
    if (nPairs > 0) {
        if (nb.group) {
            narrow_group(w, P, nPairs, nb, s, cntp);
            k_narrow<<<(nPairs + 127) / 128, 128, 0, s>>>(w, P, gridn_nb(nPairs), nb.perm, nb.blockOff,
                                                           (EpaRec*)nb.queue, nb.queueCount, nullptr); note_launch();
        } else {
            k_narrow<<<(nPairs + 127) / 128, 128, 0, s>>>(w, P, nPairs, nullptr, nullptr, (EpaRec*)nb.queue,
                                                           nb.queueCount, cntp); note_launch();
        }
    }
    if (prof) { prof->mark(PH_NARROW, 1, s); prof->mark(PH_EPA, 0, s); }
    if (nPairs > 0) epa_tiers(w, P, nb.queue, nb.queueCount, nb.ovfQueue, nb.ovfQueue2, nb.ovfCount, nb.slots, nullptr, nullptr, s);
    if (prof) prof->mark(PH_EPA, 1, s);
}

// ---- concave pass: convex objects against triangle meshes ---------------------------------
// ConvexConcaveCollisionAlgorithm.processCollision (collision/dispatch/ConvexConcaveCollision
// Algorithm.java:65-97) for every pair whose algorithm is convex-concave: the convex object's
// aabb in the mesh's space widened by the mesh margin (ConvexTriangleCallback.
// setTimeStepAndCounters, java:82-104) is quantized and the mesh's quantized tree walked
// (OptimizedBvh.walkStacklessQuantizedTree, java:940-997); each triangle found is collided by
// ConvexConvexAlgorithm as a TriangleShape with the mesh margin (ConvexTriangleCallback.
// processTriangle, java:109-166) into the pair's one manifold, then the manifold is refreshed.
// On the GPU the triangles of all pairs become (pair, triangle) candidates - counted, scanned,
// listed in walk order - whose GJK (and EPA) runs one thread (one warp) each; the points are then
// added to each pair's manifold in walk order by one thread per pair, which is what makes the
// result the reference's: a manifold's point replacement depends on the order points arrive.

// The convex object and the mesh of a convex-concave pair; false for any other pair or when
// neither body is active (needsCollision).
JBD bool concave_pair(const DevWorld& w, const DevPairs& P, int p, int& col0, int& col1, Xf& x0, Xf& x1, Leaf& c,
                      Leaf& t) {
    const uint64_t key = P.keys[p];
    const int a = key_owner(key), b = key_partner(key);
    col0 = min(a, b);
    col1 = max(a, b);
    if (!is_active_state(w.act[col0]) && !is_active_state(w.act[col1])) return false;
    int t0, t1;
    const int k = pair_leaf_types(w, key, col0, col1, t0, t1);
    if (k != ALG_CONVEX_CONCAVE && k != ALG_CONCAVE_CONVEX) return false;
    x0 = load_xf(w, col0);
    x1 = load_xf(w, col1);
    Leaf f, g;
    pair_leaves(w, key, col0, col1, x0, x1, f, g);
    c = k == ALG_CONVEX_CONCAVE ? f : g;
    t = k == ALG_CONVEX_CONCAVE ? g : f;
    return true;
}

// Per pair: the ConvexTriangleCallback's manifold on first contact, the candidate count, and the
// pair appended to the list of mesh pairs (list[0] counts them; the fill and the merge run over
// the list, a thread per mesh pair, in whatever order the appends landed - pairs are independent).
__global__ void k_mesh_count(DevWorld w, DevPairs P, int nPairs, const int* cntp, int* cnt, int* list) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPairs) return;
    int col0, col1;
    Xf x0, x1;
    Leaf c, t;
    const bool mine = p < (cntp ? min(nPairs, *cntp) : nPairs) && concave_pair(w, P, p, col0, col1, x0, x1, c, t);
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, mine);
    if (!mine) {
        cnt[p] = 0;
        return;
    }
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(list, __popc(m));
    base = __shfl_sync(m, base, leader);
    list[1 + base + __popc(m & ((1u << lane) - 1u))] = p;
    if (!P.has[p]) { P.has[p] = 1; P.n[p] = 0; }
    cnt[p] = mesh_walk(w, c, t, p, nullptr);
}

// The pair's candidates in walk order at its offset; cap: the candidate buffer's capacity (sized
// from the count pass's bound; a pair that would run past it flags ST_CAPACITY).
__global__ void k_mesh_fill(DevWorld w, DevPairs P, const int* list, const int* off, int2* cand, int cap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= list[0]) return;
    const int p = list[1 + i];
    int col0, col1;
    Xf x0, x1;
    Leaf c, t;
    concave_pair(w, P, p, col0, col1, x0, x1, c, t);
    const int room = cap - off[p];
    if (mesh_walk(w, c, t, p, cand + off[p], room) > room) atomicOr(&w.ctr[C_STATUS], ST_CAPACITY);
}

// Per candidate: GjkPairDetector between the convex object and the triangle (ConvexConvex
// Algorithm.processCollision java:90-139 with the callback's manifold); penetrating candidates
// go to the EPA queue.  res: 2 float4 per candidate (pointOnB + offset, distance; normal, valid).
__global__ void __launch_bounds__(128, 4) k_mesh_gjk(DevWorld w, DevPairs P, const int2* cand, const int* total, int cap,
                                                     float4* res, EpaRec* queue, int* queueCount) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(*total, cap)) return;
    const int2 ct = cand[i];
    int col0, col1;
    Xf x0, x1;
    Leaf c, t;
    concave_pair(w, P, ct.x, col0, col1, x0, x1, c, t);
    const ShapeRef sa = shape_ref(w.sh, c.shape), sb = triangle_ref(w.sh, t.shape, ct.y);
    float md = __fadd_rn(__fadd_rn(sa.margin, sb.margin), w.cbt);
    md = __fmul_rn(md, md);
    atomicAdd(&w.ctr[C_GJK], 1);
    const GjkPart g = gjk_part(sa, c.x, sb, t.x, md);
    if (g.needEpa) {
        EpaRec r;
        r.pair = i;
        r.valid = g.isValid ? 1 : 0;
        r.distance = g.distance;
        r.pad = 0.0f;
        r.pA = f4(g.pointOnA, 0.0f);
        r.pB = f4(g.pointOnB, 0.0f);
        r.nB = f4(g.normalInB, 0.0f);
        queue[atomicAdd(queueCount, 1)] = r;
        return;
    }
    res[2 * i] = f4(add(g.pointOnB, g.offset), g.distance);
    res[2 * i + 1] = f4(g.normalInB, g.isValid ? 1.0f : 0.0f);
}

// Per pair: the candidates' points into the manifold in walk order (ManifoldResult.
// addContactPoint), then ManifoldResult.refreshContactPoints.
__global__ void k_mesh_merge(DevWorld w, DevPairs P, const int* list, const int* cnt, const int* off,
                             const float4* res) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= list[0]) return;
    const int p = list[1 + i];
    int col0, col1;
    Xf x0, x1;
    Leaf c, t;
    concave_pair(w, P, p, col0, col1, x0, x1, c, t);
    const int mb0 = P.b0[p], mb1 = P.b1[p];
    Mf m;
    load_mf(P, p, m);
    const float fr0 = w.friction[col0], fr1 = w.friction[col1], re0 = w.restitution[col0], re1 = w.restitution[col1];
    for (int k = off[p], e = off[p] + cnt[p]; k < e; k++) {
        const float4 a = res[2 * k], b = res[2 * k + 1];
        if (b.w != 0.0f) add_contact(m, mb0, col0, x0, x1, fr0, fr1, re0, re1, mk4(b), mk4(a), a.w, w.cbt);
    }
    manifold_refresh(m, w, mb0, mb1);
    store_mf(P, p, m);
}

void concave_free(NarrowBuffers& nb) {
    cudaFree(nb.meshCnt); cudaFree(nb.meshOff); cudaFree(nb.meshTotal); cudaFree(nb.meshScan); cudaFree(nb.meshList);
    nb.meshList = nullptr;
    cudaFree(nb.cand); cudaFree(nb.candRes); cudaFree(nb.candQueue); cudaFree(nb.candOvf); cudaFree(nb.candOvf2);
    cudaFree(nb.candCount);
    nb.meshCnt = nb.meshOff = nb.meshTotal = nullptr;
    nb.meshScan = nullptr;
    nb.cand = nullptr;
    nb.candRes = nullptr;
    nb.candQueue = nullptr;
    nb.candOvf = nb.candOvf2 = nb.candCount = nullptr;
    nb.capMeshPairs = nb.capCand = 0;
}

// Buffers of the concave pass for pairCap pairs and candCap candidates (grown, never shrunk).
// Returns -1 when a CUDA allocation failed, 1 when a buffer moved (captured graphs hold the old
// pointers), 0 otherwise.
int concave_reserve(NarrowBuffers& nb, int pairCap, int candCap, cudaStream_t s) {
    int moved = 0;
    if (pairCap > nb.capMeshPairs) {
        cudaFree(nb.meshCnt); cudaFree(nb.meshOff); cudaFree(nb.meshScan); cudaFree(nb.meshList);
        nb.meshCnt = nb.meshOff = nb.meshList = nullptr;
        nb.meshScan = nullptr;
        const int c = std::max(pairCap, 2 * nb.capMeshPairs);
        if (cudaMalloc(&nb.meshCnt, sizeof(int) * c) != cudaSuccess || cudaMalloc(&nb.meshOff, sizeof(int) * c) != cudaSuccess ||
            cudaMalloc(&nb.meshList, sizeof(int) * (c + 1)) != cudaSuccess ||
            cudaMalloc(&nb.meshScan, scan_scratch_bytes(c)) != cudaSuccess)
            return -1;
        nb.capMeshPairs = c;
        moved = 1;
    }
    if (!nb.meshTotal) {
        if (cudaMalloc(&nb.meshTotal, sizeof(int)) != cudaSuccess) return -1;
        moved = 1;
    }
    if (!nb.candCount) {
        if (cudaMalloc(&nb.candCount, sizeof(int) * 4) != cudaSuccess) return -1;
        cudaMemsetAsync(nb.candCount, 0, sizeof(int) * 4, s);
        moved = 1;
    }
    if (candCap > nb.capCand || !nb.cand) {
        cudaFree(nb.cand); cudaFree(nb.candRes); cudaFree(nb.candQueue); cudaFree(nb.candOvf); cudaFree(nb.candOvf2);
        nb.cand = nullptr;
        nb.candRes = nullptr;
        nb.candQueue = nullptr;
        nb.candOvf = nb.candOvf2 = nullptr;
        const int c = std::max(std::max(candCap, 1), 2 * nb.capCand);
        if (cudaMalloc(&nb.cand, sizeof(int2) * c) != cudaSuccess || cudaMalloc(&nb.candRes, sizeof(float4) * 2 * c) != cudaSuccess ||
            cudaMalloc(&nb.candQueue, sizeof(EpaRec) * c) != cudaSuccess || cudaMalloc(&nb.candOvf, sizeof(int) * c) != cudaSuccess ||
            cudaMalloc(&nb.candOvf2, sizeof(int) * c) != cudaSuccess)
            return -1;
        nb.capCand = c;
        moved = 1;
    }
    return moved;
}

// The pass on reserved buffers with every count on the device: nPairs bounds the pair count (cntp:
// the device count, or null for exactly nPairs) and the candidate buffer holds the count pass's
// bound.  Grids are sized by the capacities; kernels read the counts.
static void concave_passes(const DevWorld& w, DevPairs& P, int nPairs, const int* cntp, NarrowBuffers& nb, cudaStream_t s,
                           bool haveCandidates) {
    const int blocks = (nPairs + 127) / 128;
    cudaMemsetAsync(nb.meshList, 0, sizeof(int), s);
    k_mesh_count<<<blocks, 128, 0, s>>>(w, P, nPairs, cntp, nb.meshCnt, nb.meshList); note_launch();
    exclusive_scan(nb.meshCnt, nb.meshOff, nb.meshTotal, nPairs, nb.meshScan, s);
    if (haveCandidates) {
        k_mesh_fill<<<blocks, 128, 0, s>>>(w, P, nb.meshList, nb.meshOff, nb.cand, nb.capCand); note_launch();
        cudaMemsetAsync(nb.candCount, 0, sizeof(int), s);
        k_mesh_gjk<<<(nb.capCand + 127) / 128, 128, 0, s>>>(w, P, nb.cand, nb.meshTotal, nb.capCand, nb.candRes,
                                                            (EpaRec*)nb.candQueue, nb.candCount);
        note_launch();
        epa_tiers(w, P, nb.candQueue, nb.candCount, nb.candOvf, nb.candOvf2, nb.candCount + 1, nb.slots, nb.cand,
                  nb.candRes, s);
    }
    k_mesh_merge<<<blocks, 128, 0, s>>>(w, P, nb.meshList, nb.meshCnt, nb.meshOff, nb.candRes); note_launch();
}

int concave_launch_bounded(const DevWorld& w, DevPairs& P, int nPairs, const int* cntp, NarrowBuffers& nb, int candBound,
                           cudaStream_t s) {
    (void)candBound;   // the buffers hold it (concave_reserve); the candidate kernels always run, so a
                       // captured graph replays for any count
    if (nPairs <= 0) return 0;
    concave_passes(w, P, nPairs, cntp, nb, s, true);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

int concave_launch(const DevWorld& w, DevPairs& P, int nPairs, const int* cntp, NarrowBuffers& nb, int* hostTotal,
                   cudaStream_t s) {
    if (nPairs <= 0) return 0;
    if (concave_reserve(nb, nPairs, 0, s) < 0) return 1;
    // the exact candidate count first (the stage path: no bound from a count pass of this step)
    cudaMemsetAsync(nb.meshList, 0, sizeof(int), s);
    k_mesh_count<<<(nPairs + 127) / 128, 128, 0, s>>>(w, P, nPairs, cntp, nb.meshCnt, nb.meshList); note_launch();
    exclusive_scan(nb.meshCnt, nb.meshOff, nb.meshTotal, nPairs, nb.meshScan, s);
    if (cudaMemcpyAsync(hostTotal, nb.meshTotal, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return 1;
    if (concave_reserve(nb, nPairs, *hostTotal, s) < 0) return 1;
    concave_passes(w, P, nPairs, cntp, nb, s, *hostTotal > 0);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

size_t epa_queue_record_bytes() { return sizeof(EpaRec); }

int narrowphase_configure() {
    return (cudaFuncSetAttribute(k_narrow_epa_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)EPA_SMEM_BYTES) ==
                cudaSuccess &&
            cudaFuncSetAttribute(EPA_T1_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)EPA_T1_SMEM_BYTES) ==
                cudaSuccess &&
            cudaFuncSetAttribute(EPA_T2_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)EPA_T2_SMEM_BYTES) ==
                cudaSuccess) ? 0 : 1;
}

// ---- EPA pass on scratch compiled into the library ----------------------------------------
// Some hosts cannot allocate device memory on the per-frame path: an engine that reserves its
// whole device budget at start-up and treats any later cudaMalloc as a failure, or a frame
// loop that cannot afford the device-wide synchronisation that cudaFree implies.  For them the
// EPA pass can take its per-slot polytope scratch from this file-scope array instead of the
// world's arena.  Size: STATIC_EPA_SLOTS (32) slots of 95.1 KiB each, 2.97 MiB in all.
// Nothing in it needs to start at zero: an EPA run writes every face, vertex, seen-ray and
// stack entry before it reads it.  One array per device, shared by every world on it, so two
// calls that overlap in time on one device (other streams or host threads) race on it.
namespace {
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t EPA_FACE_BYTES = (size_t)STATIC_EPA_SLOTS * EPA_FACE_CAP * sizeof(float4);
constexpr size_t EPA_FACED_BYTES = (size_t)STATIC_EPA_SLOTS * EPA_FACE_CAP * sizeof(float);
constexpr size_t EPA_MKV_BYTES = (size_t)STATIC_EPA_SLOTS * EPA_MKV_CAP * sizeof(float4);
constexpr size_t EPA_SEEN_BYTES = (size_t)STATIC_EPA_SLOTS * EPA_SEEN_CAP * sizeof(float4);
constexpr size_t EPA_STACK_BYTES = (size_t)STATIC_EPA_SLOTS * EPA_STACK_CAP * sizeof(int2);
// fN, fV, fF, fE | fD | mW, mR | seen | stack, each region 256-byte aligned
constexpr size_t OFF_FN = 0;
constexpr size_t OFF_FV = OFF_FN + align256(EPA_FACE_BYTES);
constexpr size_t OFF_FF = OFF_FV + align256(EPA_FACE_BYTES);
constexpr size_t OFF_FE = OFF_FF + align256(EPA_FACE_BYTES);
constexpr size_t OFF_FD = OFF_FE + align256(EPA_FACE_BYTES);
constexpr size_t OFF_MW = OFF_FD + align256(EPA_FACED_BYTES);
constexpr size_t OFF_MR = OFF_MW + align256(EPA_MKV_BYTES);
constexpr size_t OFF_SEEN = OFF_MR + align256(EPA_MKV_BYTES);
constexpr size_t OFF_STACK = OFF_SEEN + align256(EPA_SEEN_BYTES);
constexpr size_t STATIC_EPA_BYTES = OFF_STACK + align256(EPA_STACK_BYTES);
}  // namespace

static __device__ __align__(256) unsigned char g_epaScratch[STATIC_EPA_BYTES];

size_t epa_static_scratch_bytes() { return STATIC_EPA_BYTES; }

int epa_static_scratch(int device, void** base) {
    static std::mutex mu;
    static void* perDevice[MAX_STATIC_DEVICES] = {};
    if (device < 0 || device >= MAX_STATIC_DEVICES) return 1;
    std::lock_guard<std::mutex> lock(mu);
    if (!perDevice[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_epaScratch);   // the caller made `device` current
        if (e != cudaSuccess || !p) return 1;
        perDevice[device] = p;
    }
    *base = perDevice[device];
    return 0;
}

void narrowphase_launch_static(const DevWorld& w, DevPairs& P, int nPairs, NarrowBuffers& nb, void* base, int slots,
                               cudaStream_t s) {
    cudaMemsetAsync(nb.queueCount, 0, sizeof(int), s);
    if (nPairs <= 0) return;
    narrow_group(w, P, nPairs, nb, s);
    k_narrow<<<(nPairs + 127) / 128, 128, 0, s>>>(w, P, gridn_nb(nPairs), nb.perm, nb.blockOff, (EpaRec*)nb.queue,
                                                   nb.queueCount, nullptr); note_launch();
    unsigned char* b = (unsigned char*)base;
    EpaArena ar;
    ar.fN = (float4*)(b + OFF_FN);
    ar.fV = (int4*)(b + OFF_FV);
    ar.fF = (int4*)(b + OFF_FF);
    ar.fE = (int4*)(b + OFF_FE);
    ar.fD = (float*)(b + OFF_FD);
    ar.mW = (float4*)(b + OFF_MW);
    ar.mR = (float4*)(b + OFF_MR);
    ar.seen = (float4*)(b + OFF_SEEN);
    ar.stack = (int2*)(b + OFF_STACK);
    ar.slots = slots;
    k_narrow_epa<<<(slots * 32 + 127) / 128, 128, 0, s>>>(w, P, (const EpaRec*)nb.queue, nb.queueCount, ar); note_launch();
}

}  // namespace jbg
