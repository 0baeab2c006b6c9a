// Islands, sleeping and the sequential-impulse contact solver.
//
// Islands: union-find over every overlapping pair whose bodies both merge islands
// (collision/dispatch/SimulationIslandManager.java:57-105, UnionFind.java:55-143), with
// lock-free hooking of the larger root under the smaller (root = lowest body index), then
// the per-island sleep decision and the islandmanifold filter of buildIslands
// (SimulationIslandManager.java:120-240) and the skip of islands with an inactive body
// (SimulationIslandManager.java:283-296).
//
// Solver: SequentialImpulseConstraintSolver.solveGroupCacheFriendly
// (dynamics/constraintsolver/SequentialImpulseConstraintSolver.java:418-924), made parallel by
// colouring manifolds so that no two manifolds of a colour share a dynamic body.  Gauss-Seidel
// within a colour is then order-independent and the colour phases equal the reference solver
// run on the manifolds sorted by (colour, pair index), the order hook of F8
// (SequentialImpulseConstraintSolver.java:769-779).  Colouring: each round, every dynamic body
// is claimed by the lowest candidate index touching it; candidates holding all their claims
// take the round's colour.  One cooperative persistent kernel colours, another runs warm
// start, numIterations x (normal colours, friction colours) and write-back, separated by a
// bounded grid barrier.
#include <cooperative_groups.h>
#include "manifold.cuh"
#include "prims.cuh"
#include "solver.cuh"

namespace jbg {
using namespace jbd;

static inline int gridn(int n, int b) { return (n + b - 1) / b; }

// ---- islands ------------------------------------------------------------------------------
__device__ __forceinline__ int uf_find(int* parent, int x) {
    int p = __ldcg(&parent[x]);
    while (p != x) {
        int gp = __ldcg(&parent[p]);
        if (gp != p) atomicCAS(&parent[x], p, gp);   // path halving
        x = p;
        p = __ldcg(&parent[x]);
    }
    return x;
}

__global__ void k_uf_init(int n, int* parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) parent[i] = i;
}

__global__ void k_uf_union(DevWorld w, DevPairs P, int nPairs, int* parent) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPairs) return;
    uint64_t key = P.keys[p];
    int a = (int)(key >> 32), b = (int)(key & 0xffffffffu);
    if (!merges_islands(w.flags[a]) || !merges_islands(w.flags[b])) return;
    for (int it = 0; it < 1 << 20; it++) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a > b) { int t = a; a = b; b = t; }
        if (atomicCAS(&parent[b], b, a) == b) return;
    }
    atomicOr(&w.ctr[C_STATUS], ST_TIMEOUT);
}

__global__ void k_islands(DevWorld w, int* parent, int* keepAwake, int* inactive) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    int isl = is_static_or_kin(w.flags[i]) ? -1 : uf_find(parent, i);
    w.island[i] = isl;
    keepAwake[i] = 0;
    inactive[i] = 0;
}

__global__ void k_island_awake(DevWorld w, int* keepAwake) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    int isl = w.island[i];
    if (isl < 0) return;
    if (isl == i) atomicAdd(&w.ctr[C_ISLANDS], 1);
    int a = w.act[i];
    if (a == ACTIVE_TAG || a == DISABLE_DEACTIVATION) keepAwake[isl] = 1;
}

__global__ void k_island_sleep(DevWorld w, const int* keepAwake, int* inactive) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    int isl = w.island[i];
    if (isl < 0) return;
    int a = w.act[i];
    if (!keepAwake[isl]) a = set_activation(a, ISLAND_SLEEPING);
    else if (a == ISLAND_SLEEPING) a = set_activation(a, WANTS_DEACTIVATION);
    w.act[i] = a;
    if (!is_active_state(a)) inactive[isl] = 1;
}

// Candidate manifolds: in islandmanifold, island processed, at least one point with distance <= 0.
__global__ void k_select(DevWorld w, DevPairs P, int nPairs, const int* inactive, int* flag) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPairs) return;
    int f = 0;
    if (P.has[p]) {
        int b0 = P.b0[p], b1 = P.b1[p];
        int a0 = w.act[b0], a1 = w.act[b1];
        int f0 = w.flags[b0], f1 = w.flags[b1];
        bool resp = !(f0 & CF_NO_CONTACT_RESPONSE) && !(f1 & CF_NO_CONTACT_RESPONSE) &&
                    (!is_static_or_kin(f0) || !is_static_or_kin(f1));
        if ((a0 != ISLAND_SLEEPING || a1 != ISLAND_SLEEPING) && resp) {
            int isl = w.island[b0] >= 0 ? w.island[b0] : w.island[b1];
            if (!inactive[isl]) {
                int n = P.n[p];
                for (int j = 0; j < n; j++)
                    if (P.pA[p * 4 + j].w <= 0.0f) { f = 1; break; }
            }
        }
    }
    flag[p] = f;
}

__global__ void k_compact(int nPairs, const int* flag, const int* idx, int* cand) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < nPairs && flag[p]) cand[idx[p]] = p;
}

// Manifold counts (has, points) for the counters.
__global__ void k_count_manifolds(DevPairs P, int nPairs, int* ctr) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int m = 0, c = 0;
    if (p < nPairs && P.has[p]) { m = 1; c = P.n[p]; }
    for (int o = 16; o > 0; o >>= 1) { m += __shfl_down_sync(0xffffffffu, m, o); c += __shfl_down_sync(0xffffffffu, c, o); }
    if ((threadIdx.x & 31) == 0 && (m || c)) { atomicAdd(&ctr[C_MANIFOLDS], m); atomicAdd(&ctr[C_CONTACTS], c); }
}

void islands_launch(const DevWorld& w, const DevPairs& P, int nPairs, SolverBuffers& sb, cudaStream_t s) {
    int n = w.nBodies;
    k_uf_init<<<gridn(n, 256), 256, 0, s>>>(n, sb.parent); note_launch();
    if (nPairs > 0) { k_uf_union<<<gridn(nPairs, 256), 256, 0, s>>>(w, P, nPairs, sb.parent); note_launch(); }
    k_islands<<<gridn(n, 256), 256, 0, s>>>(w, sb.parent, sb.keepAwake, sb.inactive); note_launch();
    k_island_awake<<<gridn(n, 256), 256, 0, s>>>(w, sb.keepAwake); note_launch();
    k_island_sleep<<<gridn(n, 256), 256, 0, s>>>(w, sb.keepAwake, sb.inactive); note_launch();
    if (nPairs > 0) {
        k_select<<<gridn(nPairs, 256), 256, 0, s>>>(w, P, nPairs, sb.inactive, sb.flag); note_launch();
        exclusive_scan(sb.flag, sb.candIdx, sb.nCand, nPairs, sb.scanScratch, s);
        k_compact<<<gridn(nPairs, 256), 256, 0, s>>>(nPairs, sb.flag, sb.candIdx, sb.cand); note_launch();
        k_count_manifolds<<<gridn(nPairs, 256), 256, 0, s>>>(P, nPairs, w.ctr); note_launch();
    } else {
        cudaMemsetAsync(sb.nCand, 0, sizeof(int), s);
    }
}

// ---- grid barrier (bounded wait) -----------------------------------------------------------
constexpr long long BARRIER_SPIN_LIMIT = 20000000;

__device__ __forceinline__ void grid_barrier(int* ctr, int nblocks) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile int* vgen = &ctr[C_BAR_GEN];
        volatile int* vst = &ctr[C_STATUS];
        int g = *vgen;
        __threadfence();
        int arrived = atomicAdd(&ctr[C_BAR_COUNT], 1);
        if (arrived == nblocks - 1) {
            atomicExch(&ctr[C_BAR_COUNT], 0);
            __threadfence();
            atomicAdd(&ctr[C_BAR_GEN], 1);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                __nanosleep(32);
                if (++spins > BARRIER_SPIN_LIMIT || (*vst & ST_TIMEOUT)) { atomicOr(&ctr[C_STATUS], ST_TIMEOUT); break; }
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// ---- colouring (cooperative) --------------------------------------------------------------
__device__ __forceinline__ bool dyn(const DevWorld& w, int b) { return w.island[b] >= 0; }

__global__ void k_colour(DevWorld w, DevPairs P, SolverBuffers sb) {
    const int nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int nCand = *sb.nCand;
    int* rem[2] = {sb.remA, sb.remB};
    for (int k = tid; k < nCand; k += nth) rem[0][k] = k;
    for (int c = tid; c <= MAX_COLOURS; c += nth) sb.colourCount[c] = 0;
    if (tid == 0) { w.ctr[C_REMAIN0] = nCand; w.ctr[C_REMAIN1] = 0; }
    grid_barrier(w.ctr, nb);
    int round = 0;
    for (; round < MAX_COLOURS; round++) {
        int cur = round & 1;
        int nrem = __ldcg(&w.ctr[C_REMAIN0 + cur]);
        if (nrem == 0) break;
        if (tid == 0) w.ctr[C_REMAIN0 + (cur ^ 1)] = 0;
        unsigned long long tag = (unsigned long long)(MAX_COLOURS - round) << 32;
        for (int i = tid; i < nrem; i += nth) {
            int k = __ldcg(&rem[cur][i]);
            int p = sb.cand[k];
            int b0 = P.b0[p], b1 = P.b1[p];
            if (dyn(w, b0)) atomicMin(&sb.claim[b0], tag | (unsigned)k);
            if (dyn(w, b1)) atomicMin(&sb.claim[b1], tag | (unsigned)k);
        }
        grid_barrier(w.ctr, nb);
        for (int i = tid; i < nrem; i += nth) {
            int k = __ldcg(&rem[cur][i]);
            int p = sb.cand[k];
            int b0 = P.b0[p], b1 = P.b1[p];
            unsigned long long me = tag | (unsigned)k;
            bool win = (!dyn(w, b0) || __ldcg(&sb.claim[b0]) == me) && (!dyn(w, b1) || __ldcg(&sb.claim[b1]) == me);
            if (win) {
                sb.colourOf[k] = round;
                atomicAdd(&sb.colourCount[round], 1);
            } else {
                int q = atomicAdd(&w.ctr[C_REMAIN0 + (cur ^ 1)], 1);
                rem[cur ^ 1][q] = k;
            }
        }
        grid_barrier(w.ctr, nb);
    }
    if (round >= MAX_COLOURS && __ldcg(&w.ctr[C_REMAIN0 + (round & 1)]) != 0) {
        if (tid == 0) atomicOr(&w.ctr[C_STATUS], ST_CAPACITY);
        round = MAX_COLOURS;
    }
    if (tid == 0) {
        int run = 0;
        for (int c = 0; c < round; c++) { sb.colourStart[c] = run; run += __ldcg(&sb.colourCount[c]); }
        sb.colourStart[round] = run;
        *sb.nColours = round;
        w.ctr[C_COLOURS] = round;
    }
}

// Slot assignment (kept out of the cooperative kernel for clarity): slot -> pair.
__global__ void k_slots(SolverBuffers sb, DevRows rows) {
    int nCand = *sb.nCand;
    int nCol = *sb.nColours;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nCand) return;
    int c = sb.colourOf[k];
    if (c >= nCol) return;
    int slot = sb.colourStart[c] + atomicAdd(&sb.colourFill[c], 1);
    rows.slot_pair[slot] = sb.cand[k];
}

// ---- row setup (solveGroupCacheFriendlySetup, java:418-786) -------------------------------
struct BodyV { V lin, ang, com; float im; M iw; };

JBD BodyV load_body(const DevWorld& w, int b) {
    BodyV r;
    r.lin = mk4(w.linvel[b]);
    r.ang = mk4(w.angvel[b]);
    r.com = mk(w.xr0[b].w, w.xr1[b].w, w.xr2[b].w);
    r.im = w.iloc[b].w;
    r.iw = load_iw(w, b);
    return r;
}

JBD void friction_row(const DevRows& R, int fi, V dir, V rp1, V rp2, const BodyV& A, const BodyV& B, float impulse) {
    V t1 = crs(rp1, dir), t2 = crs(rp2, dir);
    V angA = mulMv(t1, A.iw), angB = mulMv(t2, B.iw);
    float d0 = __fadd_rn(A.im, dot(dir, crs(angA, rp1)));
    float d1 = __fadd_rn(B.im, dot(dir, crs(angB, rp2)));
    float jac = jdiv(1.0f, __fadd_rn(d0, d1));
    R.f_nrm[fi] = f4(dir, jac);
    R.f_rp1[fi] = f4(t1, impulse);
    R.f_rp2[fi] = f4(t2, 0.0f);
    R.f_angA[fi] = f4(angA, 0.0f);
    R.f_angB[fi] = f4(angB, 0.0f);
}

__global__ void k_setup(DevWorld w, DevPairs P, DevRows R, const int* nCandPtr, float dt) {
    int nSlots = *nCandPtr;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nSlots) return;
    int p = R.slot_pair[s];
    int b0 = P.b0[p], b1 = P.b1[p];
    BodyV A = load_body(w, b0), B = load_body(w, b1);
    const bool warm = (w.solverMode & 4) != 0;
    int n = P.n[p];
    int mask = 0;
    for (int j = 0; j < n; j++) {
        int k = p * 4 + j;
        float4 pa = P.pA[k];
        float dist = pa.w;
        if (!(dist <= 0.0f)) continue;
        mask |= 1 << j;
        float4 wa = P.wA[k], wb = P.wB[k], nr = P.nrm[k], im = P.imp[k];
        V nrm = mk(nr.x, nr.y, nr.z);
        V rp1 = sub(mk(wa.x, wa.y, wa.z), A.com), rp2 = sub(mk(wb.x, wb.y, wb.z), B.com);
        V angA = mulMv(crs(rp1, nrm), A.iw);
        V angB = mulMv(crs(rp2, nrm), B.iw);
        float d0 = __fadd_rn(A.im, dot(nrm, crs(angA, rp1)));
        float d1 = __fadd_rn(B.im, dot(nrm, crs(angB, rp2)));
        float jac = jdiv(1.0f, __fadd_rn(d0, d1));
        V rp1xn = crs(rp1, nrm), rp2xn = crs(rp2, nrm);
        V vel1 = add(crs(A.ang, rp1), A.lin);
        V vel2 = add(crs(B.ang, rp2), B.lin);
        V vel = sub(vel1, vel2);
        float rel_vel = dot(nrm, vel);
        float pen = jmin(__fadd_rn(dist, w.slop), 0.0f);
        float rest = __fmul_rn(wb.w, -rel_vel);
        if (rest <= 0.0f) rest = 0.0f;
        float penVel = jdiv(-pen, dt);
        if (rest > penVel) pen = 0.0f;
        float imp = warm ? __fmul_rn(nr.w, w.warm) : 0.0f;
        int ni = s * 4 + j;
        R.n_nrm[ni] = f4(nrm, jac);
        R.n_rp1[ni] = f4(rp1xn, pen);
        R.n_rp2[ni] = f4(rp2xn, rest);
        R.n_angA[ni] = f4(angA, wa.w);   // friction coefficient
        R.n_angB[ni] = f4(angB, imp);
        V dir1, dir2;
        if (im.z == 0.0f) {
            dir1 = sub(vel, scl(nrm, rel_vel));
            float lat = len2(dir1);
            if (lat > FLT_EPS) {
                dir1 = scl(dir1, jdiv(1.0f, jsqrt(lat)));
                dir2 = nor(crs(dir1, nrm));
            } else {
                plane_space1(nrm, dir1, dir2);
            }
            P.d1[k] = f4(dir1, 0.0f);
            P.d2[k] = f4(dir2, 0.0f);
            P.imp[k] = make_float4(im.x, im.y, 1.0f, 0.0f);
        } else {
            dir1 = mk4(P.d1[k]);
            dir2 = mk4(P.d2[k]);
        }
        friction_row(R, ni * 2 + 0, dir1, rp1, rp2, A, B, warm ? __fmul_rn(im.x, w.warm) : 0.0f);
        friction_row(R, ni * 2 + 1, dir2, rp1, rp2, A, B, warm ? __fmul_rn(im.y, w.warm) : 0.0f);
    }
    R.slot_mask[s] = mask;
    atomicAdd(&w.ctr[C_ROWS], __popc(mask));
}

// ---- PGS (cooperative) --------------------------------------------------------------------
JBD void apply_imp(V& lin, V& ang, V n, float im, V angc, float imp) {   // SolverBody.internalApplyImpulse
    if (im != 0.0f) {
        V lc = scl(n, im);
        lin.x = __fadd_rn(lin.x, __fmul_rn(imp, lc.x));
        lin.y = __fadd_rn(lin.y, __fmul_rn(imp, lc.y));
        lin.z = __fadd_rn(lin.z, __fmul_rn(imp, lc.z));
        ang.x = __fadd_rn(ang.x, __fmul_rn(imp, angc.x));
        ang.y = __fadd_rn(ang.y, __fmul_rn(imp, angc.y));
        ang.z = __fadd_rn(ang.z, __fmul_rn(imp, angc.z));
    }
}

struct Vel { V l0, a0, l1, a1; float im0, im1; };

JBD void load_vel(const DevWorld& w, int b0, int b1, Vel& v) {
    float4 t;
    t = __ldcg(&w.linvel[b0]); v.l0 = mk(t.x, t.y, t.z);
    t = __ldcg(&w.angvel[b0]); v.a0 = mk(t.x, t.y, t.z);
    t = __ldcg(&w.linvel[b1]); v.l1 = mk(t.x, t.y, t.z);
    t = __ldcg(&w.angvel[b1]); v.a1 = mk(t.x, t.y, t.z);
    v.im0 = w.iloc[b0].w;
    v.im1 = w.iloc[b1].w;
}
JBD void store_vel(const DevWorld& w, int b0, int b1, const Vel& v) {
    if (v.im0 != 0.0f) { __stcg(&w.linvel[b0], f4(v.l0, 0.0f)); __stcg(&w.angvel[b0], f4(v.a0, 0.0f)); }
    if (v.im1 != 0.0f) { __stcg(&w.linvel[b1], f4(v.l1, 0.0f)); __stcg(&w.angvel[b1], f4(v.a1, 0.0f)); }
}

__global__ void k_pgs(DevWorld w, DevPairs P, DevRows R, const int* nColoursPtr, const int* nCandPtr, float dt) {
    const int nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int nCol = *nColoursPtr;
    const int nSlots = *nCandPtr;
    // warm start, in setup order within each manifold: normal, friction 1, friction 2 per point
    for (int c = 0; c < nCol; c++) {
        int s0 = R.colour_start[c], s1 = R.colour_start[c + 1];
        for (int s = s0 + tid; s < s1; s += nth) {
            int p = R.slot_pair[s];
            int b0 = P.b0[p], b1 = P.b1[p];
            Vel v;
            load_vel(w, b0, b1, v);
            int mask = R.slot_mask[s];
            for (int j = 0; j < 4; j++) {
                if (!(mask & (1 << j))) continue;
                int ni = s * 4 + j;
                float4 nn = R.n_nrm[ni];
                V n = mk(nn.x, nn.y, nn.z);
                float imp = R.n_angB[ni].w;
                apply_imp(v.l0, v.a0, n, v.im0, mk4(R.n_angA[ni]), imp);
                apply_imp(v.l1, v.a1, n, v.im1, mk4(R.n_angB[ni]), -imp);
                for (int f = 0; f < 2; f++) {
                    int fi = ni * 2 + f;
                    V d = mk4(R.f_nrm[fi]);
                    float fimp = R.f_rp1[fi].w;
                    apply_imp(v.l0, v.a0, d, v.im0, mk4(R.f_angA[fi]), fimp);
                    apply_imp(v.l1, v.a1, d, v.im1, mk4(R.f_angB[fi]), -fimp);
                }
            }
            store_vel(w, b0, b1, v);
        }
        grid_barrier(w.ctr, nb);
    }
    for (int it = 0; it < w.numIter; it++) {
        for (int c = 0; c < nCol; c++) {      // resolveSingleCollisionCombinedCacheFriendly (java:234-284)
            int s0 = R.colour_start[c], s1 = R.colour_start[c + 1];
            for (int s = s0 + tid; s < s1; s += nth) {
                int p = R.slot_pair[s];
                int b0 = P.b0[p], b1 = P.b1[p];
                Vel v;
                load_vel(w, b0, b1, v);
                int mask = R.slot_mask[s];
                for (int j = 0; j < 4; j++) {
                    if (!(mask & (1 << j))) continue;
                    int ni = s * 4 + j;
                    float4 nn = R.n_nrm[ni], r1 = R.n_rp1[ni], r2 = R.n_rp2[ni], aA = R.n_angA[ni];
                    float4 aB = __ldcg(&R.n_angB[ni]);
                    V n = mk(nn.x, nn.y, nn.z);
                    float vel1 = __fadd_rn(dot(n, v.l0), dot(mk(r1.x, r1.y, r1.z), v.a0));
                    float vel2 = __fadd_rn(dot(n, v.l1), dot(mk(r2.x, r2.y, r2.z), v.a1));
                    float rel = __fsub_rn(vel1, vel2);
                    float posErr = jdiv(__fmul_rn(-r1.w, w.erp), dt);
                    float velErr = __fsub_rn(r2.w, rel);
                    float ni1 = __fadd_rn(__fmul_rn(posErr, nn.w), __fmul_rn(velErr, nn.w));
                    float old = aB.w;
                    float sum = __fadd_rn(old, ni1);
                    float acc = 0.0f > sum ? 0.0f : sum;
                    float d = __fsub_rn(acc, old);
                    apply_imp(v.l0, v.a0, n, v.im0, mk(aA.x, aA.y, aA.z), d);
                    apply_imp(v.l1, v.a1, n, v.im1, mk(aB.x, aB.y, aB.z), -d);
                    aB.w = acc;
                    __stcg(&R.n_angB[ni], aB);
                }
                store_vel(w, b0, b1, v);
            }
            grid_barrier(w.ctr, nb);
        }
        for (int c = 0; c < nCol; c++) {      // resolveSingleFrictionCacheFriendly (java:286-346)
            int s0 = R.colour_start[c], s1 = R.colour_start[c + 1];
            for (int s = s0 + tid; s < s1; s += nth) {
                int p = R.slot_pair[s];
                int b0 = P.b0[p], b1 = P.b1[p];
                Vel v;
                load_vel(w, b0, b1, v);
                int mask = R.slot_mask[s];
                for (int j = 0; j < 4; j++) {
                    if (!(mask & (1 << j))) continue;
                    int ni = s * 4 + j;
                    float total = __fadd_rn(__ldcg(&R.n_angB[ni]).w, 0.0f);   // appliedImpulse + appliedPushImpulse
                    float fric = R.n_angA[ni].w;
                    float limit = __fmul_rn(total, fric);
                    if (!(total > 0.0f)) continue;
                    for (int f = 0; f < 2; f++) {
                        int fi = ni * 2 + f;
                        float4 fn = R.f_nrm[fi];
                        float4 r1 = __ldcg(&R.f_rp1[fi]);
                        float4 r2 = R.f_rp2[fi];
                        V n = mk(fn.x, fn.y, fn.z);
                        float vel1 = __fadd_rn(dot(n, v.l0), dot(mk(r1.x, r1.y, r1.z), v.a0));
                        float vel2 = __fadd_rn(dot(n, v.l1), dot(mk(r2.x, r2.y, r2.z), v.a1));
                        float rel = __fsub_rn(vel1, vel2);
                        float j1 = __fmul_rn(-rel, fn.w);
                        float old = r1.w;
                        float acc = __fadd_rn(old, j1);
                        if (limit < acc) acc = limit;
                        else if (acc < -limit) acc = -limit;
                        j1 = __fsub_rn(acc, old);
                        apply_imp(v.l0, v.a0, n, v.im0, mk4(R.f_angA[fi]), j1);
                        apply_imp(v.l1, v.a1, n, v.im1, mk4(R.f_angB[fi]), -j1);
                        r1.w = acc;
                        __stcg(&R.f_rp1[fi], r1);
                    }
                }
                store_vel(w, b0, b1, v);
            }
            grid_barrier(w.ctr, nb);
        }
    }
    // write-back (java:901-912): appliedImpulse; appliedImpulseLateral1 ends as friction row 2's
    for (int s = tid; s < nSlots; s += nth) {
        int p = R.slot_pair[s];
        int mask = R.slot_mask[s];
        for (int j = 0; j < 4; j++) {
            if (!(mask & (1 << j))) continue;
            int ni = s * 4 + j, k = p * 4 + j;
            float4 nr = P.nrm[k];
            nr.w = __ldcg(&R.n_angB[ni]).w;
            P.nrm[k] = nr;
            float4 im = P.imp[k];
            im.x = __ldcg(&R.f_rp1[ni * 2 + 1]).w;
            P.imp[k] = im;
        }
    }
}

int solver_coop_blocks(bool pgs) {
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per = 0;
    if (pgs) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pgs, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_colour, 256, 0);
    if (per < 1) per = 1;
    return sms * (per < 2 ? per : 2);
}

void solve_launch(const DevWorld& w, DevPairs& P, int nPairs, DevRows& R, SolverBuffers& sb, float dt, cudaStream_t s,
                  const Prof* prof) {
    if (prof) prof->mark(PH_COLOUR, 0, s);
    if (nPairs <= 0) {
        cudaMemsetAsync(sb.nColours, 0, sizeof(int), s);
        if (prof) {
            prof->mark(PH_COLOUR, 1, s);
            prof->mark(PH_SETUP, 0, s); prof->mark(PH_SETUP, 1, s);
            prof->mark(PH_PGS, 0, s); prof->mark(PH_PGS, 1, s);
        }
        return;
    }
    cudaMemsetAsync(sb.claim, 0xff, sizeof(unsigned long long) * w.nBodies, s);
    cudaMemsetAsync(w.ctr + C_BAR_COUNT, 0, sizeof(int), s);
    {
        DevWorld wc = w;
        DevPairs pc = P;
        SolverBuffers sc = sb;
        void* args[] = {&wc, &pc, &sc};
        cudaLaunchCooperativeKernel((void*)k_colour, sb.coopBlocksColour, 256, args, 0, s); note_launch();
    }
    cudaMemsetAsync(sb.colourFill, 0, sizeof(int) * (MAX_COLOURS + 1), s);
    k_slots<<<gridn(nPairs, 256), 256, 0, s>>>(sb, R); note_launch();
    if (prof) { prof->mark(PH_COLOUR, 1, s); prof->mark(PH_SETUP, 0, s); }
    k_setup<<<gridn(nPairs, 128), 128, 0, s>>>(w, P, R, sb.nCand, dt); note_launch();
    if (prof) { prof->mark(PH_SETUP, 1, s); prof->mark(PH_PGS, 0, s); }
    cudaMemsetAsync(w.ctr + C_BAR_COUNT, 0, sizeof(int), s);
    {
        DevWorld wc = w;
        DevPairs pc = P;
        DevRows rc = R;
        const int* ncol = sb.nColours;
        const int* ncand = sb.nCand;
        float dtc = dt;
        void* args[] = {&wc, &pc, &rc, &ncol, &ncand, &dtc};
        cudaLaunchCooperativeKernel((void*)k_pgs, sb.coopBlocksPgs, 256, args, 0, s); note_launch();
    }
    if (prof) prof->mark(PH_PGS, 1, s);
}

}  // namespace jbg
