// Narrowphase: CollisionDispatcher.dispatchAllCollisionPairs for every overlapping pair
// (collision/dispatch/CollisionDispatcher.java:252-257, DefaultNearCallback.java:39-66).
//
// Pass 1 (one thread per pair): needsCollision, algorithm creation (the pair's manifold),
// then sphere-sphere (SphereSphereCollisionAlgorithm.java:73-134), convex-plane
// (ConvexPlaneCollisionAlgorithm.java:75-136) or convex-convex GJK
// (ConvexConvexAlgorithm.java:90-139), adding at most one point and refreshing the
// manifold.  Convex pairs whose GJK ends in the penetration case are queued with their
// partial GJK result.
// Pass 2 (one thread per queued pair, grid-stride over a fixed set of scratch slots):
// GJK-EPA penetration depth, the deeper-result choice of GjkPairDetector.java:260-303,
// then the same manifold update.
#include "epa.cuh"
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

__global__ void k_narrow(DevWorld w, DevPairs P, int nPairs, EpaRec* queue, int* queueCount) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPairs) return;
    uint64_t key = P.keys[p];
    int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
    int col0 = min(a, b), col1 = max(a, b);
    if (!is_active_state(w.act[col0]) && !is_active_state(w.act[col1])) return;   // needsCollision
    int s0 = w.shape[col0], s1 = w.shape[col1];
    int t0 = w.sh.type[s0], t1 = w.sh.type[s1];
    if (t0 == SHAPE_PLANE && t1 == SHAPE_PLANE) return;
    Mf m;
    if (!P.has[p]) { P.has[p] = 1; m.n = 0; }
    else load_mf(P, p, m);
    int mb0 = P.b0[p], mb1 = P.b1[p];
    Xf x0 = load_xf(w, col0), x1 = load_xf(w, col1);
    float fr0 = w.friction[col0], fr1 = w.friction[col1], re0 = w.restitution[col0], re1 = w.restitution[col1];
    if (t0 == SHAPE_SPHERE && t1 == SHAPE_SPHERE) {
        V diff = sub(x0.o, x1.o);
        float l = len(diff);
        float r0 = w.sh.margin[s0], r1 = w.sh.margin[s1];
        float rs = __fadd_rn(r0, r1);
        if (!(l > rs)) {
            float dist = __fsub_rn(l, rs);
            V n = mk(1.0f, 0.0f, 0.0f);
            if (l > FLT_EPS) n = scl(diff, jdiv(1.0f, l));
            V pos1 = add(x1.o, scl(n, r1));
            add_contact(m, mb0, col0, x0, x1, fr0, fr1, re0, re1, n, pos1, dist, w.cbt);
        }
        manifold_refresh(m, w, mb0, mb1);
    } else if (t0 == SHAPE_PLANE || t1 == SHAPE_PLANE) {
        int ci = (t1 == SHAPE_PLANE) ? col0 : col1;       // convex body (manifold body0)
        int pi = (t1 == SHAPE_PLANE) ? col1 : col0;
        Xf cx = (ci == col0) ? x0 : x1, px = (ci == col0) ? x1 : x0;
        ShapeRef cs = shape_ref(w.sh, w.shape[ci]);
        float4 pl = w.sh.plane[w.shape[pi]];
        V pn = mk(pl.x, pl.y, pl.z);
        Xf planeInConvex = xf_mul(xf_inverse(cx), px);
        Xf convexInPlane = xf_mul(xf_inverse(px), cx);
        V dir = mulMv(scl(pn, -1.0f), planeInConvex.b);
        V vtx = support_with_margin(cs, dir);
        V vtxInPlane = xf_apply(convexInPlane, vtx);
        float distance = __fsub_rn(dot(pn, vtxInPlane), pl.w);
        V proj = sub(vtxInPlane, scl(pn, distance));
        V vtxWorld = xf_apply(px, proj);
        if (distance < w.cbt) {
            V nB = mulMv(pn, px.b);
            add_contact(m, mb0, col0, x0, x1, fr0, fr1, re0, re1, nB, vtxWorld, distance, w.cbt);
        }
        manifold_refresh(m, w, mb0, mb1);
    } else {
        ShapeRef sa = shape_ref(w.sh, s0), sb = shape_ref(w.sh, s1);
        float md = __fadd_rn(__fadd_rn(sa.margin, sb.margin), w.cbt);
        md = __fmul_rn(md, md);
        atomicAdd(&w.ctr[C_GJK], 1);
        GjkPart g = gjk_part(sa, x0, sb, x1, md);
        if (g.needEpa) {
            int q = atomicAdd(queueCount, 1);
            EpaRec r;
            r.pair = p;
            r.valid = g.isValid ? 1 : 0;
            r.distance = g.distance;
            r.pad = 0.0f;
            r.pA = f4(g.pointOnA, 0.0f);
            r.pB = f4(g.pointOnB, 0.0f);
            r.nB = f4(g.normalInB, 0.0f);
            queue[q] = r;
            if (P.n[p] == 0 && m.n == 0) P.n[p] = 0;
            return;   // the EPA pass finishes this pair
        }
        if (g.isValid) add_contact(m, mb0, col0, x0, x1, fr0, fr1, re0, re1, g.normalInB, add(g.pointOnB, g.offset), g.distance, w.cbt);
        manifold_refresh(m, w, mb0, mb1);
    }
    store_mf(P, p, m);
}

__global__ void k_narrow_epa(DevWorld w, DevPairs P, const EpaRec* queue, const int* queueCount, EpaArena arena) {
    int n = *queueCount;
    int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= arena.slots) return;
    EpaSlot sl = epa_slot(arena, slot);
    for (int qi = slot; qi < n; qi += arena.slots) {
        EpaRec r = queue[qi];
        int p = r.pair;
        uint64_t key = P.keys[p];
        int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
        int col0 = min(a, b), col1 = max(a, b);
        int mb0 = P.b0[p], mb1 = P.b1[p];
        Xf x0 = load_xf(w, col0), x1 = load_xf(w, col1);
        ShapeRef sa = shape_ref(w.sh, w.shape[col0]), sb = shape_ref(w.sh, w.shape[col1]);
        V offset = scl(add(x0.o, x1.o), 0.5f);
        Xf lA = x0, lB = x1;
        lA.o = sub(lA.o, offset);
        lB.o = sub(lB.o, offset);
        bool isValid = r.valid != 0;
        float distance = r.distance;
        V pointOnB = mk4(r.pB), normalInB = mk4(r.nB);
        atomicAdd(&w.ctr[C_EPA], 1);
        V wA, wB;
        bool ovf = false;
        if (epa_pen_depth(sa, lA, sb, lB, sl, wA, wB, ovf)) {
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
        if (ovf) atomicOr(&w.ctr[C_STATUS], ST_EPA_POOL);
        Mf m;
        load_mf(P, p, m);
        if (isValid)
            add_contact(m, mb0, col0, x0, x1, w.friction[col0], w.friction[col1], w.restitution[col0], w.restitution[col1],
                        normalInB, add(pointOnB, offset), distance, w.cbt);
        manifold_refresh(m, w, mb0, mb1);
        store_mf(P, p, m);
    }
}

void narrowphase_launch(const DevWorld& w, DevPairs& P, int nPairs, NarrowBuffers& nb, cudaStream_t s,
                        const Prof* prof) {
    if (prof) prof->mark(PH_NARROW, 0, s);
    cudaMemsetAsync(nb.queueCount, 0, sizeof(int), s);
    if (nPairs > 0) { k_narrow<<<(nPairs + 127) / 128, 128, 0, s>>>(w, P, nPairs, (EpaRec*)nb.queue, nb.queueCount); note_launch(); }
    if (prof) { prof->mark(PH_NARROW, 1, s); prof->mark(PH_EPA, 0, s); }
    EpaArena ar;
    ar.fN = nb.fN; ar.fV = nb.fV; ar.fF = nb.fF; ar.fE = nb.fE; ar.fD = nb.fD;
    ar.mW = nb.mW; ar.mR = nb.mR; ar.seen = nb.seen; ar.stack = nb.stack;
    ar.slots = nb.slots;
    if (nPairs > 0) { k_narrow_epa<<<(nb.slots + 63) / 64, 64, 0, s>>>(w, P, (const EpaRec*)nb.queue, nb.queueCount, ar); note_launch(); }
    if (prof) prof->mark(PH_EPA, 1, s);
}

size_t epa_queue_record_bytes() { return sizeof(EpaRec); }

}  // namespace jbg
