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
// (dynamics/constraintsolver/SequentialImpulseConstraintSolver.java:418-924) made parallel
// without changing its arithmetic.  Gauss-Seidel over manifolds gives the same floats for any
// two manifold orders in which every pair of manifolds sharing a dynamic body keeps its relative
// order.  Dynamic bodies are split into parts (a batch world each, or ranges of the Morton leaf
// order); a manifold whose dynamic bodies lie in one part is internal to it, else cut.  Internal
// manifolds are coloured per part, cut manifolds grid-wide, so that no two manifolds of a colour
// share a dynamic body.  Every phase (warm start, then numIterations x normal rows, friction
// rows) runs the parts' local colours with their velocities in shared memory, then the cut
// colours: the reference solver run on the manifolds sorted by (part, colour) with cut
// manifolds last, the order hook of SequentialImpulseConstraintSolver.java:769-779.
#include <algorithm>
#include <cstdlib>
#include "../../include/jbgpu.h"
#include "manifold.cuh"
#include "mlp.cuh"
#include "prims.cuh"
#include "gridsync.cuh"
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

// Hooks the larger of the two roots under the smaller (bounded; a timeout sets ST_TIMEOUT).
__device__ __forceinline__ void uf_unite(int* parent, int a, int b, int* ctr) {
    for (int it = 0; it < 1 << 20; it++) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a > b) { int t = a; a = b; b = t; }
        if (atomicCAS(&parent[b], b, a) == b) return;
    }
    atomicOr(&ctr[C_STATUS], ST_TIMEOUT);
}

__global__ void k_uf_init(int n, int* parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) parent[i] = i;
}

// Unions in rounds over the pairs (sampling, as in the Afforest connected-components
// algorithm): round 0 takes the first two pairs of every owner (keys are sorted by owner),
// rounds 1 and 2 the third and the fourth, round 3 the rest; after each round every body is
// pointed at its root.
// A later round skips a pair whose bodies already point at the same root, so most pairs of a
// large island cost two loads instead of finds and hooks along deep, contended paths.  The
// partition is the same as one pass over all pairs.
constexpr int UF_ROUNDS = 4;

__global__ void k_uf_union(DevWorld w, DevPairs P, int nPairs, const int* cntp, int* parent, int round) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (cntp ? min(nPairs, *cntp) : nPairs)) return;
    uint64_t key = P.keys[p];
    int a = key_owner(key), b = key_partner(key);
    int rank = 0;               // pairs of the same owner before p, up to 4
    while (rank < UF_ROUNDS && p - rank - 1 >= 0 && key_owner(P.keys[p - rank - 1]) == a) rank++;
    if ((rank < 2 ? 0 : rank - 1) != round) return;
    if (!merges_islands(w.flags[a]) || !merges_islands(w.flags[b])) return;
    if (round > 0 && __ldcg(&parent[a]) == __ldcg(&parent[b])) return;
    uf_unite(parent, a, b, w.ctr);
}

// Joints between two dynamic bodies, at least one of them active, join their islands
// (DiscreteDynamicsWorld.calculateSimulationIslands, java:649-677).
__global__ void k_joint_union(DevWorld w, SolverBuffers sb) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= sb.J.n) return;
    const int a = sb.J.a[j], b = sb.J.b[j];
    if (b < 0 || is_static_or_kin(w.flags[a]) || is_static_or_kin(w.flags[b])) return;
    if (!is_active_state(w.act[a]) && !is_active_state(w.act[b])) return;
    uf_unite(sb.parent, a, b, w.ctr);
}

// Every body pointed at its root (between the union rounds).
__global__ void k_uf_compress(int n, int* parent) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) parent[i] = uf_find(parent, i);
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
__global__ void k_select(DevWorld w, DevPairs P, int nPairs, const int* cntp, const int* inactive, int* flag) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nPairs) return;
    if (cntp && p >= *cntp) { flag[p] = 0; return; }   // past the device pair count: not a candidate
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
__global__ void k_count_manifolds(DevPairs P, int nPairs, const int* cntp, int* ctr) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int m = 0, c = 0;
    if (p < (cntp ? min(nPairs, *cntp) : nPairs) && P.has[p]) { m = 1; c = P.n[p]; }
    for (int o = 16; o > 0; o >>= 1) { m += __shfl_down_sync(0xffffffffu, m, o); c += __shfl_down_sync(0xffffffffu, c, o); }
    if ((threadIdx.x & 31) == 0 && (m || c)) { atomicAdd(&ctr[C_MANIFOLDS], m); atomicAdd(&ctr[C_CONTACTS], c); }
}

// Unions and the awake test read only pairs, flags and activation states, none of which the
// narrowphase writes, so a step runs them beside the narrowphase on a second stream.  cntp
// (nullable): the pair count on the device, nPairs then being only an upper bound (graph
// replays, whose launches cannot know the count).
void islands_launch_unions(const DevWorld& w, const DevPairs& P, int nPairs, SolverBuffers& sb, cudaStream_t s,
                           const int* cntp) {
    int n = w.nBodies;
    k_uf_init<<<gridn(n, 256), 256, 0, s>>>(n, sb.parent); note_launch();
    if (nPairs > 0) {
        for (int r = 0; r < UF_ROUNDS; r++) {
            if (r > 0) { k_uf_compress<<<gridn(n, 256), 256, 0, s>>>(n, sb.parent); note_launch(); }
            k_uf_union<<<gridn(nPairs, 256), 256, 0, s>>>(w, P, nPairs, cntp, sb.parent, r); note_launch();
        }
    }
    if (sb.J.n > 0) { k_joint_union<<<gridn(sb.J.n, 128), 128, 0, s>>>(w, sb); note_launch(); }
    k_islands<<<gridn(n, 256), 256, 0, s>>>(w, sb.parent, sb.keepAwake, sb.inactive); note_launch();
    k_island_awake<<<gridn(n, 256), 256, 0, s>>>(w, sb.keepAwake); note_launch();
}

// Sleep decisions (they change activation states, which the narrowphase reads) and the
// manifold selection (it reads the narrowphase's points): after the narrowphase.
void islands_launch_select(const DevWorld& w, const DevPairs& P, int nPairs, SolverBuffers& sb, cudaStream_t s,
                           const int* cntp) {
    int n = w.nBodies;
    k_island_sleep<<<gridn(n, 256), 256, 0, s>>>(w, sb.keepAwake, sb.inactive); note_launch();
    if (nPairs > 0) {
        k_select<<<gridn(nPairs, 256), 256, 0, s>>>(w, P, nPairs, cntp, sb.inactive, sb.flag); note_launch();
        exclusive_scan(sb.flag, sb.candIdx, sb.nCand, nPairs, sb.scanScratch, s);
        k_compact<<<gridn(nPairs, 256), 256, 0, s>>>(nPairs, sb.flag, sb.candIdx, sb.cand); note_launch();
        k_count_manifolds<<<gridn(nPairs, 256), 256, 0, s>>>(P, nPairs, cntp, w.ctr); note_launch();
    } else {
        cudaMemsetAsync(sb.nCand, 0, sizeof(int), s);
    }
}

void islands_launch(const DevWorld& w, const DevPairs& P, int nPairs, SolverBuffers& sb, cudaStream_t s) {
    islands_launch_unions(w, P, nPairs, sb, s, nullptr);
    islands_launch_select(w, P, nPairs, sb, s, nullptr);
}

// ---- parts and buckets ---------------------------------------------------------------------
__device__ __forceinline__ bool dyn(const DevWorld& w, int b) { return w.island[b] >= 0; }

// Claim tag of candidate k in claim pass t.  Later passes carry smaller tags, so a claim left
// from an earlier pass never beats a claim of the current one.
__device__ __forceinline__ unsigned long long ctag(int t, int k) {
    return ((unsigned long long)(0x7fffffff - t) << 32) | (unsigned)k;
}

// Part of dynamic body b, or -1 when b has no position in the body order.
__device__ __forceinline__ int part_of(const DevWorld& w, const SolverBuffers& sb, int b) {
    int pos = sb.posOf[b];
    if (pos < 0) return -1;
    return sb.worldParts ? w.world[b] : (int)(((long long)pos * sb.nParts) / sb.nFinite);
}

__global__ void k_posof(SolverBuffers sb) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < sb.nFinite) sb.posOf[sb.order[s]] = s;
}

// Bucket of candidate k: the part holding all its dynamic bodies, else nParts (cut).
__global__ void k_classify(DevWorld w, DevPairs P, SolverBuffers sb) {
    int nCand = *sb.nCand;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nCand) return;
    int p = sb.cand[k];
    int b0 = P.b0[p], b1 = P.b1[p];
    bool d0 = dyn(w, b0), d1 = dyn(w, b1);
    int q0 = d0 ? part_of(w, sb, b0) : -2, q1 = d1 ? part_of(w, sb, b1) : -2;
    int q = d0 ? q0 : q1;
    if (q == -1 || (d0 && d1 && q0 != q1)) q = sb.nParts;
    sb.bucket[k] = q;
    int lb0 = 0xffff, lb1 = 0xffff;   // dynamic bodies' indices within the part (internal candidates)
    if (q < sb.nParts) {
        int ps = sb.partStart[q];
        if (d0) lb0 = sb.posOf[b0] - ps;
        if (d1) lb1 = sb.posOf[b1] - ps;
    }
    sb.candLocal[k] = lb0 | (lb1 << 16);
    const unsigned grp = __match_any_sync(__activemask(), q);   // one atomic per bucket and warp
    if ((threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&sb.bucketCount[q], __popc(grp));
}

// Fill position of a lane among the lanes of its warp with the same key: the group's leader
// takes the group's places from *ctr with one atomic.
JBD int group_take(int* ctr, int key) {
    const unsigned grp = __match_any_sync(__activemask(), key);
    const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(ctr, __popc(grp));
    base = __shfl_sync(grp, base, leader);
    return base + __popc(grp & ((1u << lane) - 1u));
}

__global__ void k_bucket_scatter(SolverBuffers sb) {
    int nCand = *sb.nCand;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nCand) return;
    int b = sb.bucket[k];
    sb.bucketList[sb.bucketStart[b] + group_take(&sb.bucketFill[b], b)] = k;
}

// Blocks take parts largest first from a shared counter (ctr[counter], cleared before the
// launch), so that one large part does not leave the other blocks idle at the end.
JBD int next_part(const DevWorld& w, const SolverBuffers& sb, int counter, int* sh) {
    __syncthreads();
    if (threadIdx.x == 0) *sh = atomicAdd(&w.ctr[counter], 1);
    __syncthreads();
    const int k = *sh;
    return k < sb.nParts ? sb.partOrder[k] : -1;
}

// ---- colouring (cooperative) ---------------------------------------------------------------
// Each colour is grown to a maximal set by claim passes: every dynamic body is claimed by the
// lowest candidate index touching it among the eligible candidates (uncoloured, no dynamic body
// taken by the colour yet); candidates holding all their claims join the colour and take their
// bodies; passes repeat until one adds nothing (at most MAX_SUB).  Manifolds internal to a part
// are coloured by the block owning the part with block barriers; cut manifolds are coloured
// grid-wide afterwards with grid barriers.
__device__ __forceinline__ bool eligible(const DevWorld& w, const DevPairs& P, const SolverBuffers& sb, int k, int mark,
                                         int& b0, int& b1) {
    if (__ldcg(&sb.colourOf[k]) >= 0) return false;
    int p = sb.cand[k];
    b0 = P.b0[p];
    b1 = P.b1[p];
    if (dyn(w, b0) && __ldcg(&sb.taken[b0]) == mark) return false;
    if (dyn(w, b1) && __ldcg(&sb.taken[b1]) == mark) return false;
    return true;
}

__device__ __forceinline__ bool holds_claims(const DevWorld& w, const SolverBuffers& sb, int b0, int b1,
                                             unsigned long long me) {
    return (!dyn(w, b0) || __ldcg(&sb.claim[b0]) == me) && (!dyn(w, b1) || __ldcg(&sb.claim[b1]) == me);
}

__global__ void __launch_bounds__(SOLVER_THREADS) k_colour(DevWorld w, DevPairs P, SolverBuffers sb) {
    unsigned barK = 0;
    const int nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int nCand = *sb.nCand;
    __shared__ int shWin, shDone, shPart;
    for (int k = tid; k < nCand; k += nth) sb.colourOf[k] = -1;
    for (int c = tid; c < sb.nParts * (MAX_LOCAL + 1); c += nth) sb.lcCount[c] = 0;
    for (int c = tid; c <= MAX_COLOURS; c += nth) sb.colourCount[c] = 0;
    if (tid == 0) { w.ctr[C_CUT_DONE] = 0; w.ctr[C_WIN0] = w.ctr[C_WIN1] = w.ctr[C_WIN2] = 0; }
    grid_barrier(w.ctr, nb, barK);
    // manifolds internal to the parts this block takes; the part's claims and taken marks live
    // in shared memory, indexed by the bodies' positions within the part
    extern __shared__ unsigned long long colSmem[];
    unsigned long long* shClaim = colSmem;
    int* shTaken = (int*)(colSmem + sb.partMax);
    constexpr int NONE = 0xffff;
    for (int part = next_part(w, sb, C_PART_NEXT0, &shPart); part >= 0; part = next_part(w, sb, C_PART_NEXT0, &shPart)) {
        const int s0 = sb.bucketStart[part], s1 = sb.bucketStart[part + 1];
        const int np = sb.partStart[part + 1] - sb.partStart[part];
        int* lc = sb.lcCount + part * (MAX_LOCAL + 1);
        for (int i = threadIdx.x; i < np; i += blockDim.x) { shClaim[i] = ~0ull; shTaken[i] = -1; }
        if (threadIdx.x == 0) shDone = 0;
        // a thread's first COL_REG candidates (k, local bodies, coloured) stay in registers
        // through all passes; a part with more candidates than COL_REG x blockDim takes the rest
        // from global memory
        int ck[COL_REG], cl[COL_REG];
        unsigned done = 0;
#pragma unroll
        for (int j = 0; j < COL_REG; j++) {
            const int i = s0 + threadIdx.x + j * (int)blockDim.x;
            ck[j] = i < s1 ? sb.bucketList[i] : -1;
            cl[j] = ck[j] >= 0 ? sb.candLocal[ck[j]] : 0;
        }
        const int sx = s0 + COL_REG * (int)blockDim.x;   // first candidate of the global path
        __syncthreads();
        int r = 0;
        for (; r < MAX_LOCAL && shDone < s1 - s0; r++) {
            for (int sub = 0; sub < MAX_SUB; sub++) {
                const int t = r * MAX_SUB + sub;
#pragma unroll
                for (int j = 0; j < COL_REG; j++) {
                    const int k = ck[j], l0 = cl[j] & 0xffff, l1 = (cl[j] >> 16) & 0xffff;
                    if (k < 0 || (done >> j & 1u) || (l0 != NONE && shTaken[l0] == r) || (l1 != NONE && shTaken[l1] == r))
                        continue;
                    if (l0 != NONE) atomicMin(&shClaim[l0], ctag(t, k));
                    if (l1 != NONE) atomicMin(&shClaim[l1], ctag(t, k));
                }
                for (int i = sx + threadIdx.x; i < s1; i += blockDim.x) {
                    const int k = sb.bucketList[i], lb = sb.candLocal[k], l0 = lb & 0xffff, l1 = (lb >> 16) & 0xffff;
                    if (__ldcg(&sb.colourOf[k]) >= 0 || (l0 != NONE && shTaken[l0] == r) || (l1 != NONE && shTaken[l1] == r))
                        continue;
                    if (l0 != NONE) atomicMin(&shClaim[l0], ctag(t, k));
                    if (l1 != NONE) atomicMin(&shClaim[l1], ctag(t, k));
                }
                if (threadIdx.x == 0) shWin = 0;
                __syncthreads();
                int myWin = 0;
#pragma unroll
                for (int j = 0; j < COL_REG; j++) {
                    const int k = ck[j], l0 = cl[j] & 0xffff, l1 = (cl[j] >> 16) & 0xffff;
                    if (k < 0 || (done >> j & 1u) || (l0 != NONE && shTaken[l0] == r) || (l1 != NONE && shTaken[l1] == r))
                        continue;
                    const unsigned long long me = ctag(t, k);
                    if ((l0 == NONE || shClaim[l0] == me) && (l1 == NONE || shClaim[l1] == me)) {
                        sb.colourOf[k] = r;
                        done |= 1u << j;
                        if (l0 != NONE) shTaken[l0] = r;
                        if (l1 != NONE) shTaken[l1] = r;
                        myWin++;
                    }
                }
                for (int i = sx + threadIdx.x; i < s1; i += blockDim.x) {
                    const int k = sb.bucketList[i], lb = sb.candLocal[k], l0 = lb & 0xffff, l1 = (lb >> 16) & 0xffff;
                    if (__ldcg(&sb.colourOf[k]) >= 0 || (l0 != NONE && shTaken[l0] == r) || (l1 != NONE && shTaken[l1] == r))
                        continue;
                    const unsigned long long me = ctag(t, k);
                    if ((l0 == NONE || shClaim[l0] == me) && (l1 == NONE || shClaim[l1] == me)) {
                        sb.colourOf[k] = r;
                        if (l0 != NONE) shTaken[l0] = r;
                        if (l1 != NONE) shTaken[l1] = r;
                        myWin++;
                    }
                }
                myWin = __reduce_add_sync(0xffffffffu, myWin);
                if ((threadIdx.x & 31) == 0 && myWin) atomicAdd(&shWin, myWin);
                __syncthreads();
                const int won = shWin;
                if (threadIdx.x == 0) {
                    shDone += won;
                    if (won) atomicAdd(&lc[r], won);
                }
                __syncthreads();
                if (won == 0) break;
            }
        }
        if (threadIdx.x == 0) {
            if (shDone < s1 - s0) atomicOr(&w.ctr[C_STATUS], ST_CAPACITY);
            sb.nLocal[part] = r;
            int* st = sb.lcStart + part * (MAX_LOCAL + 1);
            int run = s0;
            for (int c = 0; c < r; c++) { st[c] = run; run += __ldcg(&lc[c]); }
            st[r] = run;
        }
        __syncthreads();
    }
    // cut manifolds, grid-wide
    grid_barrier(w.ctr, nb, barK);
    const int c0 = sb.bucketStart[sb.nParts], c1 = sb.bucketStart[sb.nParts + 1];
    const int nCut = c1 - c0;
    // a thread's first COL_REG cut candidates (k and its dynamic bodies, -1 for a static one)
    // stay in registers through all passes; the rest come from global memory
    int gk[COL_REG], gb0[COL_REG], gb1[COL_REG];
    unsigned gdone = 0;
#pragma unroll
    for (int j = 0; j < COL_REG; j++) {
        const int i = c0 + tid + j * nth;
        gk[j] = i < c1 ? sb.bucketList[i] : -1;
        gb0[j] = gb1[j] = -1;
        if (gk[j] >= 0) {
            const int p = sb.cand[gk[j]];
            const int b0 = P.b0[p], b1 = P.b1[p];
            gb0[j] = dyn(w, b0) ? b0 : -1;
            gb1[j] = dyn(w, b1) ? b1 : -1;
        }
    }
    const int cx = c0 + COL_REG * nth;   // first candidate of the global path
    int g = 0, round = 0;
    for (; round < MAX_COLOURS; round++) {
        if (__ldcg(&w.ctr[C_CUT_DONE]) >= nCut) break;
        const int mark = (1 << 20) | round;
        for (int sub = 0; sub < MAX_SUB; sub++, g++) {
            const int t = (MAX_LOCAL + 1 + round) * MAX_SUB + sub;
            if (tid == 0) w.ctr[C_WIN0 + (g + 1) % 3] = 0;
            bool elig[COL_REG];
#pragma unroll
            for (int j = 0; j < COL_REG; j++) {
                elig[j] = gk[j] >= 0 && !(gdone >> j & 1u) && (gb0[j] < 0 || __ldcg(&sb.taken[gb0[j]]) != mark) &&
                          (gb1[j] < 0 || __ldcg(&sb.taken[gb1[j]]) != mark);
                if (!elig[j]) continue;
                if (gb0[j] >= 0) atomicMin(&sb.claim[gb0[j]], ctag(t, gk[j]));
                if (gb1[j] >= 0) atomicMin(&sb.claim[gb1[j]], ctag(t, gk[j]));
            }
            for (int i = cx + tid; i < c1; i += nth) {
                int k = sb.bucketList[i], b0, b1;
                if (!eligible(w, P, sb, k, mark, b0, b1)) continue;
                if (dyn(w, b0)) atomicMin(&sb.claim[b0], ctag(t, k));
                if (dyn(w, b1)) atomicMin(&sb.claim[b1], ctag(t, k));
            }
            grid_barrier(w.ctr, nb, barK);
            int won = 0;
#pragma unroll
            for (int j = 0; j < COL_REG; j++) {
                if (!elig[j]) continue;   // taken marks only change after this pass's check
                const unsigned long long me = ctag(t, gk[j]);
                if ((gb0[j] < 0 || __ldcg(&sb.claim[gb0[j]]) == me) && (gb1[j] < 0 || __ldcg(&sb.claim[gb1[j]]) == me)) {
                    sb.colourOf[gk[j]] = round;
                    gdone |= 1u << j;
                    if (gb0[j] >= 0) sb.taken[gb0[j]] = mark;
                    if (gb1[j] >= 0) sb.taken[gb1[j]] = mark;
                    won++;
                }
            }
            for (int i = cx + tid; i < c1; i += nth) {
                int k = sb.bucketList[i], b0, b1;
                if (!eligible(w, P, sb, k, mark, b0, b1)) continue;
                if (holds_claims(w, sb, b0, b1, ctag(t, k))) {
                    sb.colourOf[k] = round;
                    if (dyn(w, b0)) sb.taken[b0] = mark;
                    if (dyn(w, b1)) sb.taken[b1] = mark;
                    won++;
                }
            }
            won = __reduce_add_sync(0xffffffffu, won);   // one set of counter atomics per warp
            if ((threadIdx.x & 31) == 0 && won) {
                atomicAdd(&sb.colourCount[round], won);
                atomicAdd(&w.ctr[C_WIN0 + g % 3], won);
                atomicAdd(&w.ctr[C_CUT_DONE], won);
            }
            grid_barrier(w.ctr, nb, barK);
            if (__ldcg(&w.ctr[C_WIN0 + g % 3]) == 0) { g++; break; }
        }
    }
    if (tid == 0) {
        if (__ldcg(&w.ctr[C_CUT_DONE]) < nCut) atomicOr(&w.ctr[C_STATUS], ST_CAPACITY);
        int run = c0;
        for (int c = 0; c < round; c++) { sb.colourStart[c] = run; run += __ldcg(&sb.colourCount[c]); }
        sb.colourStart[round] = run;
        *sb.nColours = round;
        int maxLocal = 0;
        for (int p = 0; p < sb.nParts; p++) maxLocal = max(maxLocal, __ldcg(&sb.nLocal[p]));
        w.ctr[C_COLOURS] = round + maxLocal;
        w.ctr[C_CUT_COLOURS] = round;
        w.ctr[C_CUT_MANIFOLDS] = nCut;
    }
}

// Slot of each candidate: internal ones by (part, local colour), cut ones by colour.  Candidates
// left uncoloured (capacity exceeded, reported as an error) fill the rest of their bucket so
// that every slot below nCand names a valid pair; they are set up but never solved.
__global__ void k_slots(DevWorld w, DevPairs P, SolverBuffers sb, DevRows R) {
    int nCand = *sb.nCand;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nCand) return;
    int b = sb.bucket[k], c = sb.colourOf[k];
    int slot;
    if (b < sb.nParts) {
        int* fill = sb.lcFill + b * (MAX_LOCAL + 1);
        const int* st = sb.lcStart + b * (MAX_LOCAL + 1);
        if (c < 0) c = sb.nLocal[b];
        slot = st[c] + group_take(&fill[c], b * (MAX_LOCAL + 1) + c);
    } else {
        if (c < 0) c = *sb.nColours;
        slot = sb.colourStart[c] + group_take(&sb.colourFill[c], -1 - c);
    }
    int p = sb.cand[k];
    R.slot_pair[slot] = p;
    int b0 = P.b0[p], b1 = P.b1[p];
    int lb0 = 0xffff, lb1 = 0xffff;
    if (b < sb.nParts && sb.partSmem && sb.partStart[b + 1] - sb.partStart[b] <= sb.smemCap) {
        int ps = sb.partStart[b];
        if (dyn(w, b0)) lb0 = sb.posOf[b0] - ps;
        if (dyn(w, b1)) lb1 = sb.posOf[b1] - ps;
    }
    R.slot_desc[slot] = make_int4(b0, b1, 0, lb0 | (lb1 << 16));
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

// Points with rows (distance <= 0) of every slot: the mask into slot_desc.z and the count into
// slot_pt0 (scanned afterwards into the slot's first point row); 0 beyond the candidates.
__global__ void k_point_masks(DevPairs P, DevRows R, const int* nCandPtr, int nPairs) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nPairs) return;
    int cnt = 0;
    if (s < *nCandPtr) {
        int p = R.slot_pair[s];
        int n = P.n[p], mask = 0;
        for (int j = 0; j < n; j++)
            if (P.pA[p * 4 + j].w <= 0.0f) mask |= 1 << j;
        R.slot_desc[s].z = mask;
        cnt = __popc(mask);
    }
    R.slot_pt0[s] = cnt;
}

// slot_desc.z = first point row << 4 | point mask (after the scan of the counts).
__global__ void k_point_rows(DevRows R, const int* nCandPtr) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= *nCandPtr) return;
    int4 d = R.slot_desc[s];
    d.z = (R.slot_pt0[s] << 4) | (d.z & 15);
    R.slot_desc[s] = d;
}

// Rows are stored per point, compactly: the rows of slot s are [pt0, pt0 + popcount(mask)),
// one normal row per point and its two friction rows at 2 * row and 2 * row + 1.
__global__ void k_setup(DevWorld w, DevPairs P, DevRows R, const int* nCandPtr, float dt) {
    int nSlots = *nCandPtr;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nSlots) return;
    int p = R.slot_pair[s];
    int4 desc = R.slot_desc[s];
    BodyV A = load_body(w, desc.x), B = load_body(w, desc.y);
    const bool warm = (w.solverMode & 4) != 0;
    const int mask = desc.z & 15;
    int ni = desc.z >> 4;
    for (int j = 0; j < 4; j++) {
        if (!(mask & (1 << j))) continue;
        int k = p * 4 + j;
        float4 pa = P.pA[k];
        float dist = pa.w;
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
        R.pt_key[ni] = (s << 2) | j;
        R.n_nrm[ni] = f4(nrm, jac);
        R.n_rp1[ni] = f4(rp1xn, jdiv(__fmul_rn(-pen, w.erp), dt));   // positionalError (java:248)
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
        ++ni;
    }
    R.slot_im[s] = make_float2(A.im, B.im);
    const unsigned am = __activemask();
    const int rows = __reduce_add_sync(am, __popc(mask));
    if ((threadIdx.x & 31) == __ffs(am) - 1) atomicAdd(&w.ctr[C_ROWS], rows);
}

// ---- PGS (cooperative) ---------------------------------------------------------------------
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

enum { PH_WARM = 0, PH_NORMAL = 1, PH_FRICTION = 2 };

// Largest |delta lambda| and |lambda| a thread has seen in the current iteration (the
// residual of the residual-terminated mode).  `x > m` keeps NaN out, as the oracle does.
struct Resid {
    float d = 0.0f, l = 0.0f;
    JBD void add(float dl, float lam) {
        dl = fabsf(dl);
        lam = fabsf(lam);
        if (dl > d) d = dl;
        if (lam > l) l = lam;
    }
};

// Row loads.  Within k_pgs only the applied impulses (n_angB.w, f_rp1.w) change, and a row is
// read and written by the same thread in every phase; the other fields are read through the
// non-coherent path.  The loads are volatile so that all loads of a point issue together, ahead
// of its stores, instead of one memory round trip per row.
JBD float4 ld_ro(const float4* p) {
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}
JBD float4 ld_rw(const float4* p) {
    float4 v;
    asm volatile("ld.global.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}
JBD float ld_rw_w(const float4* p) {
    float v;
    asm volatile("ld.global.f32 %0, [%1];" : "=f"(v) : "l"((const float*)p + 3));
    return v;
}

JBD float ld_ro_w(const float4* p) {
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"((const float*)p + 3));
    return v;
}

// ---- point pool --------------------------------------------------------------------------
// The points of a manifold are solved one after another, so a manifold with k points would
// wait for k round trips to L2.  A thread that solves a manifold with more than one point
// copies the rows of its second to last points into entries of a per-block pool in shared
// memory with cp.async while it solves the first point from registers; they have arrived by
// the time it needs them.  An entry holds one point's fields of the phase: normal phase
// n_nrm, n_rp1, n_rp2, n_angA, n_angB; friction phase n_angA, n_angB and the two friction rows'
// f_nrm, f_rp1, f_rp2, f_angA, f_angB.  Two pools alternate between consecutive colours; when
// a pool is full the points are read from global memory.
constexpr int POOL_F4 = 12;
// entry size of a phase: a normal-phase entry holds 5 float4, so a pool holds 12/5 as many
JBD int pool_stride(int kind) { return kind == PH_NORMAL ? 5 : POOL_F4; }
JBD int pool_entries(int cap, int kind) { return kind == PH_NORMAL ? cap * POOL_F4 / 5 : cap; }

struct PointPool {
    float4* e = nullptr;    // this colour's pool (POOL_F4 float4 per entry)
    int* top = nullptr;     // its fill counter (shared memory)
    int cap = 0;            // entries
};
struct PoolSlot {           // the entries one manifold took: its point j >= j0 is entry j - j0
    const float4* e = nullptr;
    int j0 = 1;
    bool waited = false;
};

// A thread's slot of the next step, staged during the current one: its descriptor and inverse
// masses, and (pool permitting) all its points' rows in entries of the next step's pool.
struct Staged {
    int4 d = make_int4(0, 0, -1, 0);    // d.z < 0: nothing staged
    float2 im = make_float2(0.0f, 0.0f);
    const float4* e = nullptr;
};

JBD void cp_async16(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
JBD void cp_async_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Copies the fields of phase `kind` of points j0.. of the manifold with first-row word z into
// entries of pool pp; null when the pool has no room.
JBD float4* pool_copy(const PointPool& pp, const DevRows& R, int kind, int z, int j0) {
    const int npt = __popc(z & 15), pt0 = z >> 4;
    if (pp.cap == 0 || npt <= j0 || kind == PH_WARM) return nullptr;
    const int base = atomicAdd(pp.top, npt - j0);
    if (base + npt - j0 > pool_entries(pp.cap, kind)) return nullptr;
    const int es = pool_stride(kind);
    float4* e = pp.e + (size_t)base * es;
    for (int j = j0; j < npt; j++, e += es) {
        const int ni = pt0 + j;
        if (kind == PH_NORMAL) {
            cp_async16(e + 0, R.n_nrm + ni); cp_async16(e + 1, R.n_rp1 + ni); cp_async16(e + 2, R.n_rp2 + ni);
            cp_async16(e + 3, R.n_angA + ni); cp_async16(e + 4, R.n_angB + ni);
        } else {
            cp_async16(e + 0, R.n_angA + ni); cp_async16(e + 1, R.n_angB + ni);
            for (int f = 0; f < 2; f++) {
                const int fi = ni * 2 + f;
                cp_async16(e + 2 + 5 * f, R.f_nrm + fi); cp_async16(e + 3 + 5 * f, R.f_rp1 + fi);
                cp_async16(e + 4 + 5 * f, R.f_rp2 + fi); cp_async16(e + 5 + 5 * f, R.f_angA + fi);
                cp_async16(e + 6 + 5 * f, R.f_angB + fi);
            }
        }
    }
    return pp.e + (size_t)base * es;
}
JBD PoolSlot pool_take(const PointPool& pp, const DevRows& R, int kind, int z) {
    PoolSlot ps;
    ps.e = pool_copy(pp, R, kind, z, 1);
    return ps;
}

// The rows of one manifold for one phase, on velocities held in registers.  Warm start applies
// per point the normal, then both friction impulses (setup order, java:680-760).  Points 1.. of
// a manifold with pool entries are read from them.
template <bool TRACK>
JBD void solve_manifold(const DevWorld& w, const DevRows& R, int s, int z, int kind, V& l0, V& a0, V& l1, V& a1,
                        float im0, float im1, Resid& res, PoolSlot ps = PoolSlot()) {
    const int npt = __popc(z & 15), pt0 = z >> 4;
    for (int ni = pt0; ni < pt0 + npt; ni++) {
        const float4* pe = nullptr;     // this point's pool entry
        if (ps.e && ni - pt0 >= ps.j0) {
            if (!ps.waited) { cp_async_wait(); ps.waited = true; }
            pe = ps.e + (size_t)(ni - pt0 - ps.j0) * pool_stride(kind);
        }
        if (kind == PH_WARM) {
            float4 nn = R.n_nrm[ni];
            V n = mk(nn.x, nn.y, nn.z);
            float imp = R.n_angB[ni].w;
            apply_imp(l0, a0, n, im0, mk4(R.n_angA[ni]), imp);
            apply_imp(l1, a1, n, im1, mk4(R.n_angB[ni]), -imp);
            for (int f = 0; f < 2; f++) {
                int fi = ni * 2 + f;
                V d = mk4(R.f_nrm[fi]);
                float fimp = R.f_rp1[fi].w;
                apply_imp(l0, a0, d, im0, mk4(R.f_angA[fi]), fimp);
                apply_imp(l1, a1, d, im1, mk4(R.f_angB[fi]), -fimp);
            }
        } else if (kind == PH_NORMAL) {   // resolveSingleCollisionCombinedCacheFriendly (java:234-284)
            float4 nn, r1, r2, aA, aB;
            if (pe) {
                nn = pe[0]; r1 = pe[1]; r2 = pe[2]; aA = pe[3]; aB = pe[4];
            } else {
                nn = ld_ro(R.n_nrm + ni); r1 = ld_ro(R.n_rp1 + ni); r2 = ld_ro(R.n_rp2 + ni); aA = ld_ro(R.n_angA + ni);
                aB = ld_rw(R.n_angB + ni);
            }
            V n = mk(nn.x, nn.y, nn.z);
            float vel1 = __fadd_rn(dot(n, l0), dot(mk(r1.x, r1.y, r1.z), a0));
            float vel2 = __fadd_rn(dot(n, l1), dot(mk(r2.x, r2.y, r2.z), a1));
            float rel = __fsub_rn(vel1, vel2);
            float posErr = r1.w;          // -penetration * erp / timeStep, formed once by the setup
            float velErr = __fsub_rn(r2.w, rel);
            float ni1 = __fadd_rn(__fmul_rn(posErr, nn.w), __fmul_rn(velErr, nn.w));
            float old = aB.w;
            float sum = __fadd_rn(old, ni1);
            float acc = 0.0f > sum ? 0.0f : sum;
            float d = __fsub_rn(acc, old);
            apply_imp(l0, a0, n, im0, mk(aA.x, aA.y, aA.z), d);
            apply_imp(l1, a1, n, im1, mk(aB.x, aB.y, aB.z), -d);
            aB.w = acc;
            __stcg(&R.n_angB[ni], aB);
            if (TRACK) res.add(d, acc);
        } else {                          // resolveSingleFrictionCacheFriendly (java:286-346)
            float applied, fric;
            float4 fnv[2], r1v[2], r2v[2], fav[2], fbv[2];
            if (pe) {
                fric = pe[0].w;
                applied = pe[1].w;
                for (int f = 0; f < 2; f++) {
                    fnv[f] = pe[2 + 5 * f]; r1v[f] = pe[3 + 5 * f]; r2v[f] = pe[4 + 5 * f];
                    fav[f] = pe[5 + 5 * f]; fbv[f] = pe[6 + 5 * f];
                }
            } else {
                applied = ld_rw_w(R.n_angB + ni);
                fric = ld_ro_w(R.n_angA + ni);
                for (int f = 0; f < 2; f++) {
                    const int fi = ni * 2 + f;
                    fnv[f] = ld_ro(R.f_nrm + fi);
                    r1v[f] = ld_rw(R.f_rp1 + fi);
                    r2v[f] = ld_ro(R.f_rp2 + fi);
                    fav[f] = ld_ro(R.f_angA + fi);
                    fbv[f] = ld_ro(R.f_angB + fi);
                }
            }
            float total = __fadd_rn(applied, 0.0f);   // appliedImpulse + appliedPushImpulse
            float limit = __fmul_rn(total, fric);
            if (!(total > 0.0f)) {
                if (TRACK) {
                    res.add(0.0f, r1v[0].w);
                    res.add(0.0f, r1v[1].w);
                }
                continue;
            }
            for (int f = 0; f < 2; f++) {
                int fi = ni * 2 + f;
                const float4 fn = fnv[f];
                float4 r1 = r1v[f];
                const float4 r2 = r2v[f];
                V n = mk(fn.x, fn.y, fn.z);
                float vel1 = __fadd_rn(dot(n, l0), dot(mk(r1.x, r1.y, r1.z), a0));
                float vel2 = __fadd_rn(dot(n, l1), dot(mk(r2.x, r2.y, r2.z), a1));
                float rel = __fsub_rn(vel1, vel2);
                float j1 = __fmul_rn(-rel, fn.w);
                float old = r1.w;
                float acc = __fadd_rn(old, j1);
                if (limit < acc) acc = limit;
                else if (acc < -limit) acc = -limit;
                j1 = __fsub_rn(acc, old);
                apply_imp(l0, a0, n, im0, mk4(fav[f]), j1);
                apply_imp(l1, a1, n, im1, mk4(fbv[f]), -j1);
                r1.w = acc;
                __stcg(&R.f_rp1[fi], r1);
                if (TRACK) res.add(j1, acc);
            }
        }
    }
}

JBD void gload(const DevWorld& w, int b, V& l, V& a) {
    float4 t = __ldcg(&w.linvel[b]);
    l = mk(t.x, t.y, t.z);
    t = __ldcg(&w.angvel[b]);
    a = mk(t.x, t.y, t.z);
}
JBD void gstore(const DevWorld& w, int b, V l, V a) {
    __stcg(&w.linvel[b], f4(l, 0.0f));
    __stcg(&w.angvel[b], f4(a, 0.0f));
}

// ---- point-to-point joints ----------------------------------------------------------------
// TypedConstraint's fixed body: identity transform, no mass, no inertia, at rest.
JBD Xf joint_xf(const DevWorld& w, int b) {
    if (b >= 0) return load_xf(w, b);
    Xf t;
    t.b.r[0] = mk(1.0f, 0.0f, 0.0f);
    t.b.r[1] = mk(0.0f, 1.0f, 0.0f);
    t.b.r[2] = mk(0.0f, 0.0f, 1.0f);
    t.o = mk(0.0f, 0.0f, 0.0f);
    return t;
}

// Point2PointConstraint.buildJacobian (java:72-101) of the joints whose island is processed:
// the pivot offsets, the positional error per axis and 1/Adiag per axis (JacobianEntry.init,
// JacobianEntry.java:63-78; the port's `bJ.set(rel_pos2).crs(bJ)` crosses rel_pos2 with
// itself, so the B-side angular Jacobian is the zero vector, kept as the reference computes it).
// The solve's per-iteration recomputation of these (java:103-140) gives the same floats.
// ScalarUtil.atan2Fast (linearmath/ScalarUtil.java:43-57)
constexpr float SIMD_PI_F = 6.283185307179586232f * 0.5f;   // BulletGlobals.SIMD_PI
JBD float atan2_fast(float y, float x) {
    const float c1 = __fdiv_rn(SIMD_PI_F, 4.0f), c2 = __fmul_rn(3.0f, c1);
    const float ay = fabsf(y);
    float angle;
    if (x >= 0.0f) angle = __fsub_rn(c1, __fmul_rn(c1, jdiv(__fsub_rn(x, ay), __fadd_rn(x, ay))));
    else angle = __fsub_rn(c2, __fmul_rn(c1, jdiv(__fadd_rn(x, ay), __fsub_rn(ay, x))));
    return y < 0.0f ? -angle : angle;
}
JBD V frame_col(const float4* rows, int c) {
    return mk(c == 0 ? rows[0].x : (c == 1 ? rows[0].y : rows[0].z), c == 0 ? rows[1].x : (c == 1 ? rows[1].y : rows[1].z),
              c == 0 ? rows[2].x : (c == 1 ? rows[2].y : rows[2].z));
}
// RigidBody.computeAngularImpulseDenominator (dynamics/RigidBody.java:534-541)
JBD float ang_denom(const M& iw, V axis) { return dot(axis, mulMTv(axis, iw)); }
JBD M joint_iw(const DevWorld& w, int b) {
    M r;
    r.r[0] = r.r[1] = r.r[2] = mk(0.0f, 0.0f, 0.0f);
    if (b >= 0) r = load_iw(w, b);
    return r;
}

// HingeConstraint.buildJacobian (HingeConstraint.java:240-340): three linear rows along the
// pivots' separation and its plane space (JacobianEntry.init as for the point-to-point joint),
// the limit state from the hinge angle (getHingeAngle, java:535-555), kHinge about A's hinge
// axis, and both world hinge axes (the solve's per-iteration recomputation gives the same
// floats).  The angular JacobianEntries the reference also builds are never read by its solve.
JBD void hinge_setup(const DevWorld& w, const DevJoints& J, int j, int a, int b) {
    const int kind = J.kind[j];
    const float4* F = J.frame + 6 * j;
    const Xf xa = joint_xf(w, a), xb = joint_xf(w, b);
    const float4 la = w.iloc[a], lb = b >= 0 ? w.iloc[b] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const V iA = mk(la.x, la.y, la.z), iB = mk(lb.x, lb.y, lb.z);
    const M IA = joint_iw(w, a), IB = joint_iw(w, b);
    const V pA = xf_apply(xa, mk4(J.pivA[j])), pB = xf_apply(xb, mk4(J.pivB[j]));
    const V r1 = sub(pA, xa.o), r2 = sub(pB, xb.o);
    V n[3];
    float inv[3] = {0.0f, 0.0f, 0.0f}, depth[3] = {0.0f, 0.0f, 0.0f};
    n[0] = n[1] = n[2] = mk(0.0f, 0.0f, 0.0f);
    if (!(kind & JK_ANGULAR_ONLY)) {
        const V rel = sub(pB, pA);
        n[0] = len2(rel) > FLT_EPS ? nor(rel) : mk(1.0f, 0.0f, 0.0f);
        plane_space1(n[0], n[1], n[2]);
        const M w2A = transpose(xa.b), w2B = transpose(xb.b);
        for (int i = 0; i < 3; i++) {
            const V aJ = mulMv(crs(r1, n[i]), w2A);
            const V bJ = mulMv(crs(r2, r2), w2B);
            const V m0 = mulc(iA, aJ), m1 = mulc(iB, bJ);
            const float adiag = __fadd_rn(__fadd_rn(__fadd_rn(la.w, dot(m0, aJ)), lb.w), dot(m1, bJ));
            inv[i] = jdiv(1.0f, adiag);
            depth[i] = -dot(sub(pA, pB), n[i]);
        }
    }
    const V ref0 = mulMv(frame_col(F, 0), xa.b), ref1 = mulMv(frame_col(F, 1), xa.b);
    const V swing = mulMv(frame_col(F + 3, 1), xb.b);
    const float angle = atan2_fast(dot(swing, ref0), dot(swing, ref1));
    const float4 st = J.set[j];   // lower, upper, softness, bias
    float correction = 0.0f, sign = 0.0f;
    if (st.x < st.y) {
        if (angle <= __fmul_rn(st.x, st.z)) {
            correction = __fsub_rn(st.x, angle);
            sign = 1.0f;
        } else if (angle >= __fmul_rn(st.y, st.z)) {
            correction = __fsub_rn(st.y, angle);
            sign = -1.0f;
        }
    }
    const V axisA = mulMv(frame_col(F, 2), xa.b), axisB = mulMv(frame_col(F + 3, 2), xb.b);
    const float kHinge = jdiv(1.0f, __fadd_rn(ang_denom(IA, axisA), ang_denom(IB, axisA)));
    J.r1[j] = f4(r1, 0.0f);
    J.r2[j] = f4(r2, 0.0f);
    J.dep[j] = make_float4(depth[0], depth[1], depth[2], 0.0f);
    float4* H = J.hs + JOINT_STEP_F4 * j;
    H[0] = f4(n[0], inv[0]);
    H[1] = f4(n[1], inv[1]);
    H[2] = f4(n[2], inv[2]);
    H[3] = f4(axisA, kHinge);
    H[4] = f4(axisB, correction);
    H[5] = make_float4(sign, 0.0f, 0.0f, 0.0f);
}

// Generic6DofConstraint.matrixToEulerXYZ (Generic6DofConstraint.java:125-159): element `index` is
// row index % 3, column index / 3; atan2 and asin in double precision, rounded to float.
JBD V euler_xyz(const M& m) {
    auto e = [&](int index) { return coord(m.r[index % 3], index / 3); };
    constexpr float HALF_PI = 6.283185307179586232f * 0.25f;   // BulletGlobals.SIMD_HALF_PI
    if (e(2) < 1.0f) {
        if (e(2) > -1.0f)
            return mk((float)atan2((double)-e(5), (double)e(8)), (float)asin((double)e(2)),
                      (float)atan2((double)-e(1), (double)e(0)));
        return mk(-(float)atan2((double)e(3), (double)e(4)), -HALF_PI, 0.0f);
    }
    return mk((float)atan2((double)e(3), (double)e(4)), HALF_PI, 0.0f);
}

// Generic6DofConstraint.buildJacobian (java:275-323): calculateTransforms and calculateAngleInfo
// (relative Euler angles, the three constraint axes), calcAnchorPos, the linear rows of the
// limited axes (JacobianEntry.init with the port's zero B-side angular part), the limit state of
// each angular axis (RotationalLimitMotor.testLimitValue) and the rows of the axes whose motor or
// limit applies; accumulated impulses cleared.
JBD void d6_setup(const DevWorld& w, const DevJoints& J, int j, int a, int b) {
    const float4* F = J.frame + 6 * j;
    const float4* S = J.d6set + D6_SET_F4 * j;
    const Xf xa = joint_xf(w, a), xb = joint_xf(w, b);
    const float4 la = w.iloc[a], lb = b >= 0 ? w.iloc[b] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const V iA = mk(la.x, la.y, la.z), iB = mk(lb.x, lb.y, lb.z);
    Xf fa, fb;
    fa.b.r[0] = mk4(F[0]); fa.b.r[1] = mk4(F[1]); fa.b.r[2] = mk4(F[2]); fa.o = mk4(J.pivA[j]);
    fb.b.r[0] = mk4(F[3]); fb.b.r[1] = mk4(F[4]); fb.b.r[2] = mk4(F[5]); fb.o = mk4(J.pivB[j]);
    const Xf ca = xf_mul(xa, fa), cb = xf_mul(xb, fb);
    const V diff = euler_xyz(mulMM(m3_invert(ca.b), cb.b));
    V ax[3];
    {
        const V c0 = mk(cb.b.r[0].x, cb.b.r[1].x, cb.b.r[2].x), c2 = mk(ca.b.r[0].z, ca.b.r[1].z, ca.b.r[2].z);
        ax[1] = crs(c2, c0);
        ax[0] = crs(ax[1], c2);
        ax[2] = crs(c0, ax[1]);
    }
    const float imA = la.w, imB = lb.w;
    const float weight = imB == 0.0f ? 1.0f : jdiv(imA, __fadd_rn(imA, imB));
    const V anchor = add(scl(ca.o, weight), scl(cb.o, __fsub_rn(1.0f, weight)));
    const V r1 = sub(anchor, xa.o), r2 = sub(anchor, xb.o);
    const M w2A = transpose(xa.b), w2B = transpose(xb.b);
    const bool useA = S[0].w != 0.0f;
    const V lower = mk4(S[0]), upper = mk4(S[1]);
    float4* H = J.hs + JOINT_STEP_F4 * j;
    for (int i = 0; i < 3; i++) {
        float inv = 0.0f;
        const V n = useA ? mk(coord(ca.b.r[0], i), coord(ca.b.r[1], i), coord(ca.b.r[2], i))
                         : mk(coord(cb.b.r[0], i), coord(cb.b.r[1], i), coord(cb.b.r[2], i));
        if (coord(upper, i) >= coord(lower, i)) {
            const V aJ = mulMv(crs(r1, n), w2A);
            const V bJ = mulMv(crs(r2, r2), w2B);
            const V m0 = mulc(iA, aJ), m1 = mulc(iB, bJ);
            inv = jdiv(1.0f, __fadd_rn(__fadd_rn(__fadd_rn(la.w, dot(m0, aJ)), lb.w), dot(m1, bJ)));
        }
        H[3 + i] = f4(n, inv);
    }
    float lim[3], err[3];
    for (int i = 0; i < 3; i++) {
        const float4 s0 = S[3 + 3 * i], s2 = S[5 + 3 * i];
        const float v = coord(diff, i);
        lim[i] = 0.0f;
        err[i] = 0.0f;
        if (!(s0.x > s0.y)) {                                     // testLimitValue
            if (v < s0.x) { lim[i] = 1.0f; err[i] = __fsub_rn(v, s0.x); }
            else if (v > s0.y) { lim[i] = 2.0f; err[i] = __fsub_rn(v, s0.y); }
        }
        float inv = 0.0f;
        if (lim[i] != 0.0f || s2.y != 0.0f) {                     // needApplyTorques
            const V aJ = mulMv(ax[i], w2A);
            const V bJ = mulMv(scl(ax[i], -1.0f), w2B);
            const V m0 = mulc(iA, aJ), m1 = mulc(iB, bJ);
            inv = jdiv(1.0f, __fadd_rn(dot(m0, aJ), dot(m1, bJ)));
        }
        H[6 + i] = f4(ax[i], inv);
    }
    H[0] = f4(ca.o, 0.0f);
    H[1] = f4(cb.o, 0.0f);
    H[2] = f4(anchor, 0.0f);
    H[9] = make_float4(lim[0], err[0], lim[1], err[1]);
    H[10] = make_float4(lim[2], err[2], 0.0f, 0.0f);
    H[11] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    H[12] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    J.r1[j] = f4(r1, 0.0f);
    J.r2[j] = f4(r2, 0.0f);
}

// ConeTwistConstraint.buildJacobian (ConeTwistConstraint.java:111-265): the hinge's linear rows,
// the swing angles about A's frame axes 1 and 2 (atan2Fast damped by the "fact" factor) against
// the elliptic cone of the swing spans, the twist about the frames' x axes through
// shortestArcQuat / quatRotate (linearmath/QuaternionUtil.java:49-90).  For a swing span below
// 0.05 the reference reads a stack vector it never set; A's frame axis is used here.
JBD void cone_setup(const DevWorld& w, const DevJoints& J, int j, int a, int b) {
    const int kind = J.kind[j];
    const float4* F = J.frame + 6 * j;
    const Xf xa = joint_xf(w, a), xb = joint_xf(w, b);
    const float4 la = w.iloc[a], lb = b >= 0 ? w.iloc[b] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const V iA = mk(la.x, la.y, la.z), iB = mk(lb.x, lb.y, lb.z);
    const M IA = joint_iw(w, a), IB = joint_iw(w, b);
    const V pA = xf_apply(xa, mk4(J.pivA[j])), pB = xf_apply(xb, mk4(J.pivB[j]));
    const V r1 = sub(pA, xa.o), r2 = sub(pB, xb.o);
    float4* H = J.hs + JOINT_STEP_F4 * j;
    float depth[3] = {0.0f, 0.0f, 0.0f};
    if (!(kind & JK_ANGULAR_ONLY)) {
        V n[3];
        const V rel = sub(pB, pA);
        n[0] = len2(rel) > FLT_EPS ? nor(rel) : mk(1.0f, 0.0f, 0.0f);
        plane_space1(n[0], n[1], n[2]);
        const M w2A = transpose(xa.b), w2B = transpose(xb.b);
        for (int i = 0; i < 3; i++) {
            const V aJ = mulMv(crs(r1, n[i]), w2A);
            const V bJ = mulMv(crs(r2, r2), w2B);
            const V m0 = mulc(iA, aJ), m1 = mulc(iB, bJ);
            const float adiag = __fadd_rn(__fadd_rn(__fadd_rn(la.w, dot(m0, aJ)), lb.w), dot(m1, bJ));
            H[i] = f4(n[i], jdiv(1.0f, adiag));
            depth[i] = -dot(sub(pA, pB), n[i]);
        }
    }
    const float4 st = J.set[j], s2 = J.set2[j];   // (swing1, swing2, twist, softness), (bias, relaxation)
    const V b1Axis1 = mulMv(frame_col(F, 0), xa.b), b2Axis1 = mulMv(frame_col(F + 3, 0), xb.b);
    const V b1Axis2 = mulMv(frame_col(F, 1), xa.b), b1Axis3 = mulMv(frame_col(F, 2), xa.b);
    float swing1 = 0.0f, swing2 = 0.0f;
    const float thresh = 10.0f;
    if (st.x >= 0.05f) {
        const float swx = dot(b2Axis1, b1Axis1), swy = dot(b2Axis1, b1Axis2);
        swing1 = atan2_fast(swy, swx);
        float fact = __fmul_rn(__fmul_rn(__fadd_rn(__fmul_rn(swy, swy), __fmul_rn(swx, swx)), thresh), thresh);
        fact = jdiv(fact, __fadd_rn(fact, 1.0f));
        swing1 = __fmul_rn(swing1, fact);
    }
    if (st.y >= 0.05f) {
        const float swx = dot(b2Axis1, b1Axis1), swy = dot(b2Axis1, b1Axis3);
        swing2 = atan2_fast(swy, swx);
        float fact = __fmul_rn(__fmul_rn(__fadd_rn(__fmul_rn(swy, swy), __fmul_rn(swx, swx)), thresh), thresh);
        fact = jdiv(fact, __fadd_rn(fact, 1.0f));
        swing2 = __fmul_rn(swing2, fact);
    }
    const float r1sq = jdiv(1.0f, __fmul_rn(st.x, st.x)), r2sq = jdiv(1.0f, __fmul_rn(st.y, st.y));
    const float ellipse = __fadd_rn(__fmul_rn(fabsf(__fmul_rn(swing1, swing1)), r1sq), __fmul_rn(fabsf(__fmul_rn(swing2, swing2)), r2sq));
    V swingAxis = mk(0.0f, 0.0f, 0.0f), twistAxis = mk(0.0f, 0.0f, 0.0f);
    float kSwing = 0.0f, kTwist = 0.0f, swingCorr = 0.0f, twistCorr = 0.0f, solveSwing = 0.0f, solveTwist = 0.0f;
    if (ellipse > 1.0f) {
        swingCorr = __fsub_rn(ellipse, 1.0f);
        solveSwing = 1.0f;
        const V t = add(scl(b1Axis2, dot(b2Axis1, b1Axis2)), scl(b1Axis3, dot(b2Axis1, b1Axis3)));
        swingAxis = scl(nor(crs(b2Axis1, t)), dot(b2Axis1, b1Axis1) >= 0.0f ? 1.0f : -1.0f);
        kSwing = jdiv(1.0f, __fadd_rn(ang_denom(IA, swingAxis), ang_denom(IB, swingAxis)));
    }
    if (st.z >= 0.0f) {
        const V b2Axis2 = mulMv(frame_col(F + 3, 1), xb.b);
        const V c = crs(b2Axis1, b1Axis1);
        const float d = dot(b2Axis1, b1Axis1);
        Q q;
        if ((double)d < -1.0 + (double)FLT_EPS) { q.x = 0.0f; q.y = 1.0f; q.z = 0.0f; q.w = 0.0f; }
        else {
            const float sq = jsqrt(__fmul_rn(__fadd_rn(1.0f, d), 2.0f));
            const float rs = jdiv(1.0f, sq);
            q.x = __fmul_rn(c.x, rs); q.y = __fmul_rn(c.y, rs); q.z = __fmul_rn(c.z, rs); q.w = __fmul_rn(sq, 0.5f);
        }
        const V v = b2Axis2;
        Q qw;
        qw.x = __fsub_rn(__fadd_rn(__fmul_rn(q.w, v.x), __fmul_rn(q.y, v.z)), __fmul_rn(q.z, v.y));
        qw.y = __fsub_rn(__fadd_rn(__fmul_rn(q.w, v.y), __fmul_rn(q.z, v.x)), __fmul_rn(q.x, v.z));
        qw.z = __fsub_rn(__fadd_rn(__fmul_rn(q.w, v.z), __fmul_rn(q.x, v.y)), __fmul_rn(q.y, v.x));
        qw.w = __fsub_rn(__fsub_rn(__fmul_rn(-q.x, v.x), __fmul_rn(q.y, v.y)), __fmul_rn(q.z, v.z));
        Q inv;
        inv.x = -q.x; inv.y = -q.y; inv.z = -q.z; inv.w = q.w;
        const Q r = qmul(qw, inv);
        const V ref = mk(r.x, r.y, r.z);
        const float twist = atan2_fast(dot(ref, b1Axis3), dot(ref, b1Axis2));
        const float lff = st.z > 0.05f ? st.w : 0.0f;
        if (twist <= __fmul_rn(-st.z, lff)) {
            twistCorr = -__fadd_rn(twist, st.z);
            solveTwist = 1.0f;
            twistAxis = scl(nor(scl(add(b2Axis1, b1Axis1), 0.5f)), -1.0f);
            kTwist = jdiv(1.0f, __fadd_rn(ang_denom(IA, twistAxis), ang_denom(IB, twistAxis)));
        } else if (twist > __fmul_rn(st.z, lff)) {
            twistCorr = __fsub_rn(twist, st.z);
            solveTwist = 1.0f;
            twistAxis = nor(scl(add(b2Axis1, b1Axis1), 0.5f));
            kTwist = jdiv(1.0f, __fadd_rn(ang_denom(IA, twistAxis), ang_denom(IB, twistAxis)));
        }
    }
    (void)s2;
    H[3] = f4(swingAxis, kSwing);
    H[4] = f4(twistAxis, kTwist);
    H[5] = make_float4(swingCorr, twistCorr, solveSwing, solveTwist);
    H[6] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    J.r1[j] = f4(r1, 0.0f);
    J.r2[j] = f4(r2, 0.0f);
    J.dep[j] = make_float4(depth[0], depth[1], depth[2], 0.0f);
}

// SliderConstraint.buildJacobianInt (SliderConstraint.java:465-526) with testLinLimits (714-730)
// and testAngLimits (732-756).  The bodies' roles swap when useLinearReferenceFrameA is false
// (buildJacobian, java:175-182): "A" is then the joint's body B with frame B.
JBD void slider_setup(const DevWorld& w, const DevJoints& J, int j, int a, int b) {
    const bool useA = J.set[j].x != 0.0f;
    const int ia = useA ? a : b, ib = useA ? b : a;
    const float4* F = J.frame + 6 * j + (useA ? 0 : 3);
    const float4* G = J.frame + 6 * j + (useA ? 3 : 0);
    const float4* P = J.d6set + D6_SET_F4 * j;   // 28 parameters
    const Xf xa = joint_xf(w, ia), xb = joint_xf(w, ib);
    const float4 la = ia >= 0 ? w.iloc[ia] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 lb = ib >= 0 ? w.iloc[ib] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const V iA = mk(la.x, la.y, la.z), iB = mk(lb.x, lb.y, lb.z);
    const M IA = joint_iw(w, ia), IB = joint_iw(w, ib);
    Xf fa, fb;
    fa.b.r[0] = mk4(F[0]); fa.b.r[1] = mk4(F[1]); fa.b.r[2] = mk4(F[2]); fa.o = mk4(useA ? J.pivA[j] : J.pivB[j]);
    fb.b.r[0] = mk4(G[0]); fb.b.r[1] = mk4(G[1]); fb.b.r[2] = mk4(G[2]); fb.o = mk4(useA ? J.pivB[j] : J.pivA[j]);
    const Xf ca = xf_mul(xa, fa), cb = xf_mul(xb, fb);
    auto colv = [](const M& m, int c) { return mk(coord(m.r[0], c), coord(m.r[1], c), coord(m.r[2], c)); };
    const V axis = colv(ca.b, 0);
    const V delta = sub(cb.o, ca.o);
    const float ad = dot(axis, delta);
    const V proj = mk(__fadd_rn(ca.o.x, __fmul_rn(ad, axis.x)), __fadd_rn(ca.o.y, __fmul_rn(ad, axis.y)),
                      __fadd_rn(ca.o.z, __fmul_rn(ad, axis.z)));
    const V relA = sub(proj, xa.o), relB = sub(cb.o, xb.o);
    const M w2A = transpose(xa.b), w2B = transpose(xb.b);
    float4* H = J.hs + JOINT_STEP_F4 * j;
    float depth[3];
    for (int i = 0; i < 3; i++) {
        const V n = colv(ca.b, i);
        const V aJ = mulMv(crs(relA, n), w2A);
        const V bJ = mulMv(crs(relB, relB), w2B);
        const V m0 = mulc(iA, aJ), m1 = mulc(iB, bJ);
        const float adiag = __fadd_rn(__fadd_rn(__fadd_rn(la.w, dot(m0, aJ)), lb.w), dot(m1, bJ));
        H[i] = f4(n, jdiv(1.0f, adiag));
        depth[i] = dot(delta, n);
    }
    const float lowerLin = P[0].x, upperLin = P[0].y, lowerAng = P[0].z, upperAng = P[0].w;
    float solveLin = 0.0f;
    if (lowerLin <= upperLin) {
        if (depth[0] > upperLin) { depth[0] = __fsub_rn(depth[0], upperLin); solveLin = 1.0f; }
        else if (depth[0] < lowerLin) { depth[0] = __fsub_rn(depth[0], lowerLin); solveLin = 1.0f; }
        else depth[0] = 0.0f;
    } else {
        depth[0] = 0.0f;
    }
    float angDepth = 0.0f, solveAng = 0.0f;
    if (lowerAng <= upperAng) {
        const V a0 = colv(ca.b, 1), a1 = colv(ca.b, 2), b0 = colv(cb.b, 1);
        const float rot = (float)atan2((double)dot(b0, a1), (double)dot(b0, a0));
        if (rot < lowerAng) { angDepth = __fsub_rn(rot, lowerAng); solveAng = 1.0f; }
        else if (rot > upperAng) { angDepth = __fsub_rn(rot, upperAng); solveAng = 1.0f; }
    }
    const float kAngle = jdiv(1.0f, __fadd_rn(ang_denom(IA, axis), ang_denom(IB, axis)));
    H[3] = f4(relA, depth[0]);
    H[4] = f4(relB, depth[1]);
    H[5] = f4(axis, depth[2]);
    H[6] = f4(colv(cb.b, 0), kAngle);
    H[7] = make_float4(solveLin, angDepth, solveAng, 0.0f);
    H[8] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void k_joint_setup(DevWorld w, SolverBuffers sb) {
    const DevJoints& J = sb.J;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J.n) return;
    const int a = J.a[j], b = J.b[j];
    const int ta = w.island[a], tb = b >= 0 ? w.island[b] : -1;
    const int isl = ta >= 0 ? ta : tb;
    const int on = isl >= 0 && !sb.inactive[isl];
    J.act[j] = on;
    if (!on) return;
    J.imp[j] = 0.0f;
    if ((J.kind[j] & JK_TYPE) == JOINT_HINGE) {
        hinge_setup(w, J, j, a, b);
        return;
    }
    if ((J.kind[j] & JK_TYPE) == JOINT_6DOF) {
        d6_setup(w, J, j, a, b);
        return;
    }
    if ((J.kind[j] & JK_TYPE) == JOINT_CONE) {
        cone_setup(w, J, j, a, b);
        return;
    }
    if ((J.kind[j] & JK_TYPE) == JOINT_SLIDER) {
        slider_setup(w, J, j, a, b);
        return;
    }
    const Xf xa = joint_xf(w, a), xb = joint_xf(w, b);
    const float4 la = w.iloc[a], lb = b >= 0 ? w.iloc[b] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const V iA = mk(la.x, la.y, la.z), iB = mk(lb.x, lb.y, lb.z);
    const V pA = xf_apply(xa, mk4(J.pivA[j])), pB = xf_apply(xb, mk4(J.pivB[j]));
    const V r1 = sub(pA, xa.o), r2 = sub(pB, xb.o);
    const M w2A = transpose(xa.b), w2B = transpose(xb.b);
    float inv[3], depth[3];
    V n = mk(0.0f, 0.0f, 0.0f);
    for (int i = 0; i < 3; i++) {
        set_coord(n, i, 1.0f);
        const V aJ = mulMv(crs(r1, n), w2A);
        const V bJ = mulMv(crs(r2, r2), w2B);
        const V m0 = mulc(iA, aJ), m1 = mulc(iB, bJ);
        const float adiag = __fadd_rn(__fadd_rn(__fadd_rn(la.w, dot(m0, aJ)), lb.w), dot(m1, bJ));
        inv[i] = jdiv(1.0f, adiag);
        depth[i] = -dot(sub(pA, pB), n);
        set_coord(n, i, 0.0f);
    }
    J.r1[j] = f4(r1, inv[0]);
    J.r2[j] = f4(r2, inv[1]);
    J.dep[j] = make_float4(depth[0], depth[1], depth[2], inv[2]);
}

// RigidBody.applyImpulse (dynamics/RigidBody.java:401-417) on velocities held in registers.
JBD void body_impulse(V& lin, V& ang, float im, const M& iw, V impulse, V relPos) {
    if (im == 0.0f) return;
    lin = add(lin, scl(impulse, im));
    ang = add(ang, mulMv(crs(relPos, impulse), iw));
}

// Point2PointConstraint.solveConstraint (java:103-171) of joint j on the bodies' velocities in
// global memory: per axis, impulse = depth tau / dt / Adiag - damping relVel / Adiag, clamped,
// applied to both bodies.
JBD void joint_solve(const DevWorld& w, const DevJoints& J, int j, float dt) {
    const int a = J.a[j], b = J.b[j];
    const float4 q1 = J.r1[j], q2 = J.r2[j], dp = J.dep[j], st = J.set[j];
    const V r1 = mk(q1.x, q1.y, q1.z), r2 = mk(q2.x, q2.y, q2.z);
    V vA, wA, vB = mk(0.0f, 0.0f, 0.0f), wB = mk(0.0f, 0.0f, 0.0f);
    gload(w, a, vA, wA);
    if (b >= 0) gload(w, b, vB, wB);
    const float imA = w.iloc[a].w, imB = b >= 0 ? w.iloc[b].w : 0.0f;
    const M IA = load_iw(w, a);
    M IB;
    IB.r[0] = IB.r[1] = IB.r[2] = mk(0.0f, 0.0f, 0.0f);
    if (b >= 0) IB = load_iw(w, b);
    float acc = __ldcg(J.imp + j);
    V n = mk(0.0f, 0.0f, 0.0f);
    for (int i = 0; i < 3; i++) {
        set_coord(n, i, 1.0f);
        const float inv = i == 0 ? q1.w : (i == 1 ? q2.w : dp.w);
        const float depth = i == 0 ? dp.x : (i == 1 ? dp.y : dp.z);
        const V vel = sub(add(crs(wA, r1), vA), add(crs(wB, r2), vB));   // getVelocityInLocalPoint
        const float relVel = dot(n, vel);
        float impulse = __fsub_rn(__fmul_rn(jdiv(__fmul_rn(depth, st.x), dt), inv), __fmul_rn(__fmul_rn(st.y, relVel), inv));
        if (st.z > 0.0f) {
            if (impulse < -st.z) impulse = -st.z;
            if (impulse > st.z) impulse = st.z;
        }
        acc = __fadd_rn(acc, impulse);
        const V iv = scl(n, impulse);
        body_impulse(vA, wA, imA, IA, iv, r1);
        body_impulse(vB, wB, imB, IB, scl(iv, -1.0f), r2);
        set_coord(n, i, 0.0f);
    }
    if (imA != 0.0f) gstore(w, a, vA, wA);
    if (b >= 0 && imB != 0.0f) gstore(w, b, vB, wB);
    __stcg(J.imp + j, acc);
}

// RigidBody.applyTorqueImpulse (dynamics/RigidBody.java:405-411).  A body without mass has a
// zero inverse inertia: the reference adds a zero vector, here it is skipped.
JBD void torque_impulse(V& ang, float im, const M& iw, V t) {
    if (im == 0.0f) return;
    ang = add(ang, mulMv(t, iw));
}

// HingeConstraint.solveConstraint (HingeConstraint.java:342-533) of joint j on the bodies'
// velocities in global memory: the linear rows (tau 0.3, the pivots' relative velocity taken once
// before the three rows), then the angular part on the angular velocities as they stand after
// them: the relative angular velocity orthogonal to the hinge axes and the axes' misalignment
// removed by torque impulses, the limit with its clamped accumulated impulse, the motor clipped
// per solve.
JBD void hinge_solve(const DevWorld& w, const DevJoints& J, int j, float dt) {
    const int a = J.a[j], b = J.b[j], kind = J.kind[j];
    V vA, wA, vB = mk(0.0f, 0.0f, 0.0f), wB = mk(0.0f, 0.0f, 0.0f);
    gload(w, a, vA, wA);
    if (b >= 0) gload(w, b, vB, wB);
    const float imA = w.iloc[a].w, imB = b >= 0 ? w.iloc[b].w : 0.0f;
    const M IA = load_iw(w, a), IB = joint_iw(w, b);
    const float4* H = J.hs + JOINT_STEP_F4 * j;
    float acc = __ldcg(J.imp + j);
    if (!(kind & JK_ANGULAR_ONLY)) {
        const float4 q1 = J.r1[j], q2 = J.r2[j], dp = J.dep[j];
        const V r1 = mk(q1.x, q1.y, q1.z), r2 = mk(q2.x, q2.y, q2.z);
        const V vel = sub(add(crs(wA, r1), vA), add(crs(wB, r2), vB));
        for (int i = 0; i < 3; i++) {
            const float4 h = H[i];
            const V n = mk(h.x, h.y, h.z);
            const float depth = i == 0 ? dp.x : (i == 1 ? dp.y : dp.z);
            const float relVel = dot(n, vel);
            const float impulse = __fsub_rn(__fmul_rn(jdiv(__fmul_rn(depth, 0.3f), dt), h.w), __fmul_rn(relVel, h.w));
            acc = __fadd_rn(acc, impulse);
            const V iv = scl(n, impulse);
            body_impulse(vA, wA, imA, IA, iv, r1);
            body_impulse(vB, wB, imB, IB, scl(iv, -1.0f), r2);
        }
    }
    const float4 ha = H[3], hb = H[4], hl = __ldcg(H + 5);
    const V axisA = mk(ha.x, ha.y, ha.z), axisB = mk(hb.x, hb.y, hb.z);
    const float kHinge = ha.w;
    const float4 st = J.set[j], s2 = J.set2[j];   // (lower, upper, softness, bias), (relaxation, target, max impulse)
    const V angVelA = wA, angVelB = wB;
    const V aroundA = scl(axisA, dot(axisA, angVelA)), aroundB = scl(axisB, dot(axisB, angVelB));
    V vro = sub(sub(angVelA, aroundA), sub(angVelB, aroundB));
    if (len(vro) > 0.00001f) {
        const V n = nor(vro);
        const float denom = __fadd_rn(ang_denom(IA, n), ang_denom(IB, n));
        vro = scl(vro, __fmul_rn(jdiv(1.0f, denom), s2.x));
    }
    V err = scl(scl(crs(axisA, axisB), -1.0f), jdiv(1.0f, dt));
    if (len(err) > 0.00001f) {
        const V n2 = nor(err);
        const float denom2 = __fadd_rn(ang_denom(IA, n2), ang_denom(IB, n2));
        err = scl(err, __fmul_rn(jdiv(1.0f, denom2), 1.0f));
    }
    torque_impulse(wA, imA, IA, add(scl(vro, -1.0f), err));
    torque_impulse(wB, imB, IB, sub(vro, err));
    float accLimit = hl.y;
    if (hl.x != 0.0f) {   // solveLimit
        const float amplitude = __fmul_rn(__fadd_rn(__fmul_rn(dot(sub(angVelB, angVelA), axisA), s2.x),
                                                    __fmul_rn(__fmul_rn(hb.w, jdiv(1.0f, dt)), st.w)), hl.x);
        float impulseMag = __fmul_rn(amplitude, kHinge);
        const float temp = accLimit;
        accLimit = jmax(__fadd_rn(accLimit, impulseMag), 0.0f);
        impulseMag = __fsub_rn(accLimit, temp);
        const V imp = scl(axisA, __fmul_rn(impulseMag, hl.x));
        torque_impulse(wA, imA, IA, imp);
        torque_impulse(wB, imB, IB, scl(imp, -1.0f));
    }
    if (kind & JK_MOTOR) {
        const V zero = mk(0.0f, 0.0f, 0.0f);
        const float projRelVel = dot(sub(aroundA, aroundB), axisA);
        const float unclipped = __fmul_rn(kHinge, __fsub_rn(s2.y, projRelVel));
        float clipped = unclipped > s2.z ? s2.z : unclipped;
        clipped = clipped < -s2.z ? -s2.z : clipped;
        const V motorImp = scl(axisA, clipped);
        torque_impulse(wA, imA, IA, add(motorImp, zero));
        torque_impulse(wB, imB, IB, sub(scl(motorImp, -1.0f), zero));
    }
    if (imA != 0.0f) gstore(w, a, vA, wA);
    if (b >= 0 && imB != 0.0f) gstore(w, b, vB, wB);
    __stcg(J.imp + j, acc);
    __stcg(&J.hs[JOINT_STEP_F4 * j + 5].y, accLimit);
}


// Generic6DofConstraint.solveConstraint (java:325-365): TranslationalLimitMotor.solveLinearAxis
// (TranslationalLimitMotor.java:70-150) per limited linear axis, on the velocities as the earlier
// axes left them, then RotationalLimitMotor.solveAngularLimits (RotationalLimitMotor.java:135-203)
// per angular axis whose limit or motor applies.
JBD void d6_solve(const DevWorld& w, const DevJoints& J, int j, float dt) {
    const int a = J.a[j], b = J.b[j];
    V vA, wA, vB = mk(0.0f, 0.0f, 0.0f), wB = mk(0.0f, 0.0f, 0.0f);
    gload(w, a, vA, wA);
    if (b >= 0) gload(w, b, vB, wB);
    const float imA = w.iloc[a].w, imB = b >= 0 ? w.iloc[b].w : 0.0f;
    const M IA = load_iw(w, a), IB = joint_iw(w, b);
    const float4* S = J.d6set + D6_SET_F4 * j;
    float4* H = J.hs + JOINT_STEP_F4 * j;
    const V pA = mk4(H[0]), pB = mk4(H[1]);
    const float4 q1 = J.r1[j], q2 = J.r2[j];
    const V r1 = mk(q1.x, q1.y, q1.z), r2 = mk(q2.x, q2.y, q2.z);
    const V lower = mk4(S[0]), upper = mk4(S[1]);
    const float softness = S[1].w, damping = S[2].x, restitution = S[2].y;
    float4 accL = __ldcg(H + 11), accA = __ldcg(H + 12);
    for (int i = 0; i < 3; i++) {
        if (!(coord(upper, i) >= coord(lower, i))) continue;
        const float4 h = H[3 + i];
        const V axis = mk(h.x, h.y, h.z);
        const V vel = sub(add(crs(wA, r1), vA), add(crs(wB, r2), vB));
        const float relVel = dot(axis, vel);
        float depth = -dot(sub(pA, pB), axis);
        float lo = -1e30f, hi = 1e30f;
        const float minLimit = coord(lower, i), maxLimit = coord(upper, i);
        if (minLimit < maxLimit) {
            if (depth > maxLimit) { depth = __fsub_rn(depth, maxLimit); lo = 0.0f; }
            else if (depth < minLimit) { depth = __fsub_rn(depth, minLimit); hi = 0.0f; }
            else continue;
        }
        float ni = __fmul_rn(__fmul_rn(softness, __fsub_rn(jdiv(__fmul_rn(restitution, depth), dt), __fmul_rn(damping, relVel))),
                             h.w);
        const float old = i == 0 ? accL.x : (i == 1 ? accL.y : accL.z);
        const float sum = __fadd_rn(old, ni);
        const float acc = sum > hi ? 0.0f : (sum < lo ? 0.0f : sum);
        if (i == 0) accL.x = acc; else if (i == 1) accL.y = acc; else accL.z = acc;
        ni = __fsub_rn(acc, old);
        const V iv = scl(axis, ni);
        body_impulse(vA, wA, imA, IA, iv, r1);
        body_impulse(vB, wB, imB, IB, scl(iv, -1.0f), r2);
    }
    const float4 l01 = H[9], l2 = H[10];
    for (int i = 0; i < 3; i++) {
        const float4 s0 = S[3 + 3 * i], s1 = S[4 + 3 * i], s2 = S[5 + 3 * i];
        const float lim = i == 0 ? l01.x : (i == 1 ? l01.z : l2.x);
        const float err = i == 0 ? l01.y : (i == 1 ? l01.w : l2.y);
        if (lim == 0.0f && s2.y == 0.0f) continue;                // needApplyTorques
        const float4 h = H[6 + i];
        const V axis = mk(h.x, h.y, h.z);
        float target = s0.z, maxForce = s0.w;
        if (lim != 0.0f) {
            target = jdiv(__fmul_rn(-s1.w, err), dt);
            maxForce = s1.x;
        }
        maxForce = __fmul_rn(maxForce, dt);
        const float relVel = dot(axis, sub(wA, wB));
        const float mrv = __fmul_rn(s1.z, __fsub_rn(target, __fmul_rn(s1.y, relVel)));
        if (mrv < FLT_EPS && mrv > -FLT_EPS) continue;
        const float unclipped = __fmul_rn(__fmul_rn(__fadd_rn(1.0f, s2.x), mrv), h.w);
        float clipped;
        if (unclipped > 0.0f) clipped = unclipped > maxForce ? maxForce : unclipped;
        else clipped = unclipped < -maxForce ? -maxForce : unclipped;
        const float old = i == 0 ? accA.x : (i == 1 ? accA.y : accA.z);
        const float sum = __fadd_rn(old, clipped);
        const float acc = sum > 1e30f ? 0.0f : (sum < -1e30f ? 0.0f : sum);
        if (i == 0) accA.x = acc; else if (i == 1) accA.y = acc; else accA.z = acc;
        clipped = __fsub_rn(acc, old);
        const V mi = scl(axis, clipped);
        torque_impulse(wA, imA, IA, mi);
        torque_impulse(wB, imB, IB, scl(mi, -1.0f));
    }
    if (imA != 0.0f) gstore(w, a, vA, wA);
    if (b >= 0 && imB != 0.0f) gstore(w, b, vB, wB);
    __stcg(H + 11, accL);
    __stcg(H + 12, accA);
}

// ConeTwistConstraint.solveConstraint (ConeTwistConstraint.java:267-368): the hinge's linear rows,
// then the swing and twist limits with clamped accumulated impulses, both from the angular
// velocities as the linear rows left them.
JBD void cone_solve(const DevWorld& w, const DevJoints& J, int j, float dt) {
    const int a = J.a[j], b = J.b[j], kind = J.kind[j];
    V vA, wA, vB = mk(0.0f, 0.0f, 0.0f), wB = mk(0.0f, 0.0f, 0.0f);
    gload(w, a, vA, wA);
    if (b >= 0) gload(w, b, vB, wB);
    const float imA = w.iloc[a].w, imB = b >= 0 ? w.iloc[b].w : 0.0f;
    const M IA = load_iw(w, a), IB = joint_iw(w, b);
    float4* H = J.hs + JOINT_STEP_F4 * j;
    float acc = __ldcg(J.imp + j);
    if (!(kind & JK_ANGULAR_ONLY)) {
        const float4 q1 = J.r1[j], q2 = J.r2[j], dp = J.dep[j];
        const V r1 = mk(q1.x, q1.y, q1.z), r2 = mk(q2.x, q2.y, q2.z);
        const V vel = sub(add(crs(wA, r1), vA), add(crs(wB, r2), vB));
        for (int i = 0; i < 3; i++) {
            const float4 h = H[i];
            const V n = mk(h.x, h.y, h.z);
            const float depth = i == 0 ? dp.x : (i == 1 ? dp.y : dp.z);
            const float impulse = __fsub_rn(__fmul_rn(jdiv(__fmul_rn(depth, 0.3f), dt), h.w), __fmul_rn(dot(n, vel), h.w));
            acc = __fadd_rn(acc, impulse);
            const V iv = scl(n, impulse);
            body_impulse(vA, wA, imA, IA, iv, r1);
            body_impulse(vB, wB, imB, IB, scl(iv, -1.0f), r2);
        }
    }
    const float4 s2 = J.set2[j], fl = H[5];
    float4 lim = __ldcg(H + 6);
    const V angVelA = wA, angVelB = wB;
    for (int k = 0; k < 2; k++) {
        if ((k == 0 ? fl.z : fl.w) == 0.0f) continue;
        const float4 ax = H[3 + k];
        const V axis = mk(ax.x, ax.y, ax.z);
        const float corr = k == 0 ? fl.x : fl.y;
        const float amplitude = __fadd_rn(__fmul_rn(__fmul_rn(dot(sub(angVelB, angVelA), axis), s2.y), s2.y),
                                          __fmul_rn(__fmul_rn(corr, jdiv(1.0f, dt)), s2.x));
        float mag = __fmul_rn(amplitude, ax.w);
        const float temp = k == 0 ? lim.x : lim.y;
        const float nacc = jmax(__fadd_rn(temp, mag), 0.0f);
        if (k == 0) lim.x = nacc; else lim.y = nacc;
        mag = __fsub_rn(nacc, temp);
        const V imp = scl(axis, mag);
        torque_impulse(wA, imA, IA, imp);
        torque_impulse(wB, imB, IB, scl(imp, -1.0f));
    }
    if (imA != 0.0f) gstore(w, a, vA, wA);
    if (b >= 0 && imB != 0.0f) gstore(w, b, vB, wB);
    __stcg(J.imp + j, acc);
    __stcg(H + 6, lim);
}

// SliderConstraint.solveConstraintInt (SliderConstraint.java:528-685) on the bodies in the roles
// the setup gave them.
JBD void slider_solve(const DevWorld& w, const DevJoints& J, int j, float dt) {
    const bool useA = J.set[j].x != 0.0f;
    const int ia = useA ? J.a[j] : J.b[j], ib = useA ? J.b[j] : J.a[j];
    V vA = mk(0.0f, 0.0f, 0.0f), wA = vA, vB = vA, wB = vA;
    if (ia >= 0) gload(w, ia, vA, wA);
    if (ib >= 0) gload(w, ib, vB, wB);
    const float imA = ia >= 0 ? w.iloc[ia].w : 0.0f, imB = ib >= 0 ? w.iloc[ib].w : 0.0f;
    const M IA = joint_iw(w, ia), IB = joint_iw(w, ib);
    const float4* P = J.d6set + D6_SET_F4 * j;
    float4* H = J.hs + JOINT_STEP_F4 * j;
    // parameters: [0] limits, then (soft, rest, damp) of dir lin, dir ang, lim lin, lim ang, ortho lin,
    // ortho ang from float 4, then lin motor (on, target, max), ang motor (on, target, max)
    const float* p = &P[0].x;
    auto soft = [&](int k) { return p[4 + 3 * k]; };
    auto rest = [&](int k) { return p[5 + 3 * k]; };
    auto damp = [&](int k) { return p[6 + 3 * k]; };
    const float4 h3 = H[3], h4 = H[4], h5 = H[5], h6 = H[6], h7 = H[7];
    const V relA = mk(h3.x, h3.y, h3.z), relB = mk(h4.x, h4.y, h4.z);
    const float depthv[3] = {h3.w, h4.w, h5.w};
    float4 acc = __ldcg(H + 8);
    const V vel = sub(add(crs(wA, relA), vA), add(crs(wB, relB), vB));
    for (int i = 0; i < 3; i++) {
        const float4 h = H[i];
        const V n = mk(h.x, h.y, h.z);
        const float relVel = dot(n, vel);
        const int k = i != 0 ? 4 : (h7.x != 0.0f ? 2 : 0);
        float ni = __fmul_rn(__fmul_rn(soft(k), __fsub_rn(jdiv(__fmul_rn(rest(k), depthv[i]), dt), __fmul_rn(damp(k), relVel))),
                             h.w);
        V iv = scl(n, ni);
        body_impulse(vA, wA, imA, IA, iv, relA);
        body_impulse(vB, wB, imB, IB, scl(iv, -1.0f), relB);
        if (p[22] != 0.0f && i == 0 && acc.x < p[24]) {
            ni = __fmul_rn(-__fadd_rn(p[23], relVel), h.w);
            float newAcc = __fadd_rn(acc.x, fabsf(ni));
            if (newAcc > p[24]) newAcc = p[24];
            const float del = __fsub_rn(newAcc, acc.x);
            ni = ni < 0.0f ? -del : del;
            acc.x = newAcc;
            iv = scl(n, ni);
            body_impulse(vA, wA, imA, IA, iv, relA);
            body_impulse(vB, wB, imB, IB, scl(iv, -1.0f), relB);
        }
    }
    const V axisA = mk(h5.x, h5.y, h5.z), axisB = mk(h6.x, h6.y, h6.z);
    const float kAngle = h6.w;
    const V angVelA = wA, angVelB = wB;
    const V aroundA = scl(axisA, dot(axisA, angVelA)), aroundB = scl(axisB, dot(axisB, angVelB));
    V vro = sub(sub(angVelA, aroundA), sub(angVelB, aroundB));
    if (len(vro) > 0.00001f) {
        const V n = nor(vro);
        const float denom = __fadd_rn(ang_denom(IA, n), ang_denom(IB, n));
        vro = scl(vro, __fmul_rn(__fmul_rn(jdiv(1.0f, denom), damp(5)), soft(5)));
    }
    V err = scl(crs(axisA, axisB), jdiv(1.0f, dt));
    if (len(err) > 0.00001f) {
        const V n2 = nor(err);
        const float denom2 = __fadd_rn(ang_denom(IA, n2), ang_denom(IB, n2));
        err = scl(err, __fmul_rn(__fmul_rn(jdiv(1.0f, denom2), rest(5)), soft(5)));
    }
    torque_impulse(wA, imA, IA, add(scl(vro, -1.0f), err));
    torque_impulse(wB, imB, IB, sub(vro, err));
    const int k = h7.z != 0.0f ? 3 : 1;
    float mag = __fadd_rn(__fmul_rn(dot(sub(angVelB, angVelA), axisA), damp(k)), jdiv(__fmul_rn(h7.y, rest(k)), dt));
    mag = __fmul_rn(mag, __fmul_rn(kAngle, soft(k)));
    const V imp = scl(axisA, mag);
    torque_impulse(wA, imA, IA, imp);
    torque_impulse(wB, imB, IB, scl(imp, -1.0f));
    if (p[25] != 0.0f && acc.y < p[27]) {
        const float projRelVel = dot(sub(aroundA, aroundB), axisA);
        float ai = __fmul_rn(kAngle, __fsub_rn(p[26], projRelVel));
        float newAcc = __fadd_rn(acc.y, fabsf(ai));
        if (newAcc > p[27]) newAcc = p[27];
        const float del = __fsub_rn(newAcc, acc.y);
        ai = ai < 0.0f ? -del : del;
        acc.y = newAcc;
        const V mi = scl(axisA, ai);
        torque_impulse(wA, imA, IA, mi);
        torque_impulse(wB, imB, IB, scl(mi, -1.0f));
    }
    if (ia >= 0 && imA != 0.0f) gstore(w, ia, vA, wA);
    if (ib >= 0 && imB != 0.0f) gstore(w, ib, vB, wB);
    __stcg(H + 8, acc);
}

// write-back (java:901-912): appliedImpulse; appliedImpulseLateral1 ends as friction row 2's
JBD void writeback_slot(const DevPairs& P, const DevRows& R, int s) {
    int p = R.slot_pair[s];
    int z = R.slot_desc[s].z, mask = z & 15;
    int ni = z >> 4;
    for (int j = 0; j < 4; j++) {
        if (!(mask & (1 << j))) continue;
        int k = p * 4 + j;
        float4 nr = P.nrm[k];
        nr.w = __ldcg(&R.n_angB[ni]).w;
        P.nrm[k] = nr;
        float4 im = P.imp[k];
        im.x = __ldcg(&R.f_rp1[ni * 2 + 1]).w;
        P.imp[k] = im;
        ++ni;
    }
}

struct PartView {
    int ps, np, nLoc;
    const int* lcs;
};

JBD PartView part_view(const SolverBuffers& sb, int part) {
    PartView v;
    v.ps = sb.partStart[part];
    v.np = sb.partStart[part + 1] - v.ps;
    v.nLoc = sb.nLocal[part];
    v.lcs = sb.lcStart + part * (MAX_LOCAL + 1);
    return v;
}

// Velocities of the part's bodies to shared memory and back (static and kinematic bodies are
// never written).
JBD void stage_in(const DevWorld& w, const SolverBuffers& sb, const PartView& v, float4* sl, float4* sa) {
    for (int i = threadIdx.x; i < v.np; i += blockDim.x) {
        int b = sb.order[v.ps + i];
        sl[i] = __ldcg(&w.linvel[b]);
        sa[i] = __ldcg(&w.angvel[b]);
    }
}
JBD void stage_out(const DevWorld& w, const SolverBuffers& sb, const PartView& v, const float4* sl, const float4* sa) {
    for (int i = threadIdx.x; i < v.np; i += blockDim.x) {
        int b = sb.order[v.ps + i];
        if (w.iloc[b].w != 0.0f) { __stcg(&w.linvel[b], sl[i]); __stcg(&w.angvel[b], sa[i]); }
    }
}

// Residual bookkeeping of one manifold (residual mode): skipped once its island converged,
// else its largest |delta lambda| and |lambda| of this iteration kept per slot.
struct ResCtl {
    bool on = false;        // residual-terminated mode
    bool skipConv = false;  // an island convergence test has run (iteration >= 2)
};
JBD bool res_skip(const SolverBuffers& sb, const ResCtl& rc, int s) {
    return rc.on && rc.skipConv && __ldcg(&sb.islConv[sb.slotIsl[s]]) != 0;
}
JBD void res_keep(const SolverBuffers& sb, const ResCtl& rc, int kind, int s, const Resid& r) {
    if (!rc.on || kind == PH_WARM) return;
    if (kind == PH_NORMAL) {
        __stcg(&sb.md[s], r.d);
        __stcg(&sb.ml[s], r.l);
    } else {
        float d = __ldcg(&sb.md[s]), l = __ldcg(&sb.ml[s]);
        if (r.d > d) __stcg(&sb.md[s], r.d);
        if (r.l > l) __stcg(&sb.ml[s], r.l);
    }
}

// One local colour of a part: its manifolds share no dynamic body; the part's bodies are in
// shared memory (global memory when the part does not fit).
// st: this thread's first slot of the colour, staged by the previous step (d.z < 0: not
// staged); on return, its slot sn of the next step (sn >= s1n: none), staged into poolNext.
JBD void local_colour(const DevWorld& w, const DevRows& R, const SolverBuffers& sb, int s0, int s1, int kind, bool smem,
                      float4* sl, float4* sa, const ResCtl& rc, int sn, int s1n, int kindn, const PointPool& pool,
                      const PointPool& poolNext, Staged& st) {
    int4 dn = make_int4(0, 0, -1, 0);
    float2 imn = make_float2(0.0f, 0.0f);
    if (sn < s1n) { dn = R.slot_desc[sn]; imn = R.slot_im[sn]; }
    for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
        const bool pre = s == s0 + (int)threadIdx.x && st.d.z >= 0;
        if (res_skip(sb, rc, s)) {
            if (pre && st.e) cp_async_wait();   // staged copies complete before the pool is reused
            continue;
        }
        const int4 d = pre ? st.d : R.slot_desc[s];
        const float2 im = pre ? st.im : R.slot_im[s];
        PoolSlot ps;
        if (pre && st.e) { ps.e = st.e; ps.j0 = 0; }
        else ps = pool_take(pool, R, kind, d.z);
        const int lb0 = d.w & 0xffff, lb1 = (d.w >> 16) & 0xffff;
        const bool m0 = smem && lb0 != 0xffff, m1 = smem && lb1 != 0xffff;
        V l0, a0, l1, a1;
        if (m0) { l0 = mk4(sl[lb0]); a0 = mk4(sa[lb0]); } else gload(w, d.x, l0, a0);
        if (m1) { l1 = mk4(sl[lb1]); a1 = mk4(sa[lb1]); } else gload(w, d.y, l1, a1);
        Resid res;
        if (rc.on) solve_manifold<true>(w, R, s, d.z, kind, l0, a0, l1, a1, im.x, im.y, res, ps);
        else solve_manifold<false>(w, R, s, d.z, kind, l0, a0, l1, a1, im.x, im.y, res, ps);
        res_keep(sb, rc, kind, s, res);
        if (im.x != 0.0f) { if (m0) { sl[lb0] = f4(l0, 0.0f); sa[lb0] = f4(a0, 0.0f); } else gstore(w, d.x, l0, a0); }
        if (im.y != 0.0f) { if (m1) { sl[lb1] = f4(l1, 0.0f); sa[lb1] = f4(a1, 0.0f); } else gstore(w, d.y, l1, a1); }
    }
    st.d = dn;
    st.im = imn;
    st.e = dn.z >= 0 ? pool_copy(poolNext, R, kindn, dn.z, 0) : nullptr;
}

JBD bool resid_done(float dmax, float lmax, float tol) { return jdiv(dmax, lmax > 1e-6f ? lmax : 1e-6f) <= tol; }

// Island residuals after an iteration: one warp per chunk of up to ISL_CHUNK slots of an
// island.  An island of one chunk is decided by its warp; a larger one combines its chunks'
// maxima with atomics, and the warp that finishes its last chunk decides (and clears the
// accumulators for the next iteration).  Unconverged islands are counted in ctr[flag].
constexpr int ISL_CHUNK = 1024;

JBD void island_residuals(const DevWorld& w, const SolverBuffers& sb, int flag, int it) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    const int nChunks = *sb.nIslChunks;
    for (int ch = gw; ch < nChunks; ch += nw) {
        const int2 cd = sb.islChunk[ch];
        const int isl = cd.x;
        if (__ldcg(&sb.islConv[isl])) continue;
        const int i0 = sb.islStart[isl], i1 = sb.islStart[isl + 1];
        const int e0 = i0 + cd.y * ISL_CHUNK, e1 = min(e0 + ISL_CHUNK, i1);
        Resid r;
        for (int e = e0 + lane; e < e1; e += 32) {
            const int s = sb.islList[e];
            r.add(__ldcg(&sb.md[s]), __ldcg(&sb.ml[s]));
        }
        for (int o = 16; o > 0; o >>= 1) {
            float od = __shfl_xor_sync(0xffffffffu, r.d, o), ol = __shfl_xor_sync(0xffffffffu, r.l, o);
            if (od > r.d) r.d = od;
            if (ol > r.l) r.l = ol;
        }
        if (lane != 0) continue;
        if (it <= JBGPU_RESIDUAL_TRACE_MAX) {   // the trace: maxima over every row still tested
            atomicMax(&sb.resTrace[2 * (it - 1)], __float_as_uint(r.d));
            atomicMax(&sb.resTrace[2 * (it - 1) + 1], __float_as_uint(r.l));
        }
        float dm = r.d, lm = r.l;
        const int nch = (i1 - i0 + ISL_CHUNK - 1) / ISL_CHUNK;
        if (nch > 1) {
            atomicMax((unsigned*)&sb.islAcc[2 * isl], __float_as_uint(dm));
            atomicMax((unsigned*)&sb.islAcc[2 * isl + 1], __float_as_uint(lm));
            __threadfence();
            if (atomicAdd(&sb.islDone[isl], 1) != nch - 1) continue;
            __threadfence();
            dm = __uint_as_float((unsigned)__ldcg(&sb.islAcc[2 * isl]));
            lm = __uint_as_float((unsigned)__ldcg(&sb.islAcc[2 * isl + 1]));
            sb.islAcc[2 * isl] = 0;
            sb.islAcc[2 * isl + 1] = 0;
            sb.islDone[isl] = 0;
        }
        if (resid_done(dm, lm, w.resTol)) sb.islConv[isl] = it;
        else atomicAdd(&w.ctr[flag], 1);
    }
}

// Phases: warm start, then iterations of (normal rows, friction rows): numIterations of them,
// or, with a residual tolerance, until every island's residual is within it (at most maxIter;
// the rows of an island stop once it converges).  Within a phase the parts' internal
// manifolds run first (parts share no dynamic body), then the cut colours.  With fixed
// iterations and no cut manifold every part runs all phases on its own, with no grid barrier.
__global__ void __launch_bounds__(SOLVER_THREADS, 2) k_pgs(DevWorld w, DevPairs P, DevRows R, SolverBuffers sb, float dt) {
    unsigned barK = 0;
    extern __shared__ float4 smv[];
    const int nb = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int nCut = *sb.nColours;
    const int nSlots = *sb.nCand;
    const bool smem = sb.partSmem != 0;
    float4* sl = smv;
    float4* sa = smv + sb.smemCap;
    // Three pools rotate over the colour steps: step c takes entries of pool c % 3 for its
    // manifolds' later points and stages its next slots into pool (c + 1) % 3; thread 0 clears
    // the counter of pool (c + 2) % 3 at the start of step c (its last users finished step c - 1,
    // its next users stage at the end of step c + 1, after step c's barrier).
    __shared__ int shPoolTop[3];
    float4* poolBase = smv + (smem ? 2 * sb.smemCap : 0);
    auto pool = [&](int c) {
        PointPool pp;
        pp.cap = sb.poolPts;
        pp.e = poolBase + (size_t)(c % 3) * sb.poolPts * POOL_F4;
        pp.top = &shPoolTop[c % 3];
        return pp;
    };
    if (threadIdx.x < 3) shPoolTop[threadIdx.x] = 0;
    const bool byRes = w.resTol > 0.0f;
    const int maxIt = byRes ? w.maxIter : w.numIter;
    // cut slot i of a colour goes to block i % gridDim.x, so a colour's manifolds spread over
    // every SM instead of filling the first blocks
    const int spread = threadIdx.x * gridDim.x + blockIdx.x;
    ResCtl rc;
    rc.on = byRes;
    int step = 0;           // colour steps this block has run (the pool alternates with it)
    if (nCut == 0 && !byRes && sb.J.n == 0) {
        __shared__ int shPart;
        int itMax = 0;
        for (int part = next_part(w, sb, C_PART_NEXT1, &shPart); part >= 0; part = next_part(w, sb, C_PART_NEXT1, &shPart)) {
            const PartView v = part_view(sb, part);
            const bool psm = smem && v.np <= sb.smemCap;
            if (psm) stage_in(w, sb, v, sl, sa);
            __syncthreads();
            // (small world parts: the next steps' slots are not staged, their pools are too small
            // for a block's manifolds and staging measured slower there)
            const int nl = v.nLoc;
            Staged st;
            auto run = [&](int kind, int c) {
                if (threadIdx.x == 0) shPoolTop[(step + 2) % 3] = 0;
                local_colour(w, R, sb, v.lcs[c], v.lcs[c + 1], kind, psm, sl, sa, rc, 0, 0, kind, pool(step),
                             pool(step + 1), st);
                __syncthreads();
                ++step;
            };
            for (int c = 0; c < nl; c++) run(PH_WARM, c);
            int it = 0;
            for (; it < maxIt && nl > 0; it++) {
                for (int c = 0; c < nl; c++) run(PH_NORMAL, c);
                for (int c = 0; c < nl; c++) run(PH_FRICTION, c);
            }
            if (it > itMax) itMax = it;
            if (psm) stage_out(w, sb, v, sl, sa);
            for (int s = sb.bucketStart[part] + threadIdx.x; s < sb.bucketStart[part + 1]; s += blockDim.x)
                writeback_slot(P, R, s);
            __syncthreads();
        }
        if (threadIdx.x == 0 && itMax > 0) atomicMax(&w.ctr[C_PGS_ITERS], itMax);
        return;
    }
    if (nSlots == 0 && sb.J.n == 0) return;
    const bool contacts = nSlots > 0;   // else only joints (the colouring did not run this step)
    if (tid == 0) for (int k = 0; k < 3; k++) w.ctr[C_RES0 + k] = 0;
    Staged st;
    int it = -1;          // -1: the warm-start phase
    for (;;) {
        for (int sub = 0; sub < (it < 0 ? 1 : 2); sub++) {
            const int kind = it < 0 ? PH_WARM : (sub == 0 ? PH_NORMAL : PH_FRICTION);
            if (kind == PH_NORMAL && sb.J.n > 0) {
                // the joints of processed islands, before the iteration's contact rows
                // (SequentialImpulseConstraintSolver.java:823-842), colour by colour
                for (int c = 0; c < sb.J.nCol; c++) {
                    const int j0 = sb.J.colStart[c], j1 = sb.J.colStart[c + 1];
                    for (int q = j0 + spread; q < j1; q += nth) {
                        const int j = sb.J.order[q];
                        if (!sb.J.act[j]) continue;
                        const int jt = sb.J.kind[j] & JK_TYPE;
                        if (jt == JOINT_HINGE) hinge_solve(w, sb.J, j, dt);
                        else if (jt == JOINT_6DOF) d6_solve(w, sb.J, j, dt);
                        else if (jt == JOINT_CONE) cone_solve(w, sb.J, j, dt);
                        else if (jt == JOINT_SLIDER) slider_solve(w, sb.J, j, dt);
                        else joint_solve(w, sb.J, j, dt);
                    }
                    grid_barrier(w.ctr, nb, barK);
                }
            }
            if (!contacts) continue;
            for (int part = blockIdx.x; part < sb.nParts; part += gridDim.x) {
                const PartView v = part_view(sb, part);
                const bool psm = smem && v.np <= sb.smemCap;
                if (psm) stage_in(w, sb, v, sl, sa);
                __syncthreads();
                st = Staged();
                const bool lastPart = part + (int)gridDim.x >= sb.nParts;
                for (int c = 0; c < v.nLoc; c++) {
                    // after the last colour of the block's last part: its slot in cut colour 0
                    const bool last = c + 1 == v.nLoc;
                    const bool toCut = last && lastPart && nCut > 0;
                    const int sn = last ? (toCut ? sb.colourStart[0] + spread : 0) : v.lcs[c + 1] + (int)threadIdx.x;
                    const int s1n = last ? (toCut ? sb.colourStart[1] : 0) : v.lcs[c + 2];
                    if (threadIdx.x == 0) shPoolTop[(step + 2) % 3] = 0;
                    local_colour(w, R, sb, v.lcs[c], v.lcs[c + 1], kind, psm, sl, sa, rc, sn, s1n, kind, pool(step),
                                 pool(step + 1), st);
                    __syncthreads();
                    ++step;
                }
                if (psm) stage_out(w, sb, v, sl, sa);
                __syncthreads();
            }
            grid_barrier(w.ctr, nb, barK);
            for (int c = 0; c < nCut; c++) {
                const int s0 = sb.colourStart[c], s1 = sb.colourStart[c + 1];
                // this thread's slot of the next cut colour, loaded now and staged at the end
                int4 dn = make_int4(0, 0, -1, 0);
                float2 imn = make_float2(0.0f, 0.0f);
                if (c + 1 < nCut && sb.colourStart[c + 1] + spread < sb.colourStart[c + 2]) {
                    dn = R.slot_desc[sb.colourStart[c + 1] + spread];
                    imn = R.slot_im[sb.colourStart[c + 1] + spread];
                }
                if (threadIdx.x == 0) shPoolTop[(step + 2) % 3] = 0;
                const PointPool pp = pool(step);
                for (int s = s0 + spread; s < s1; s += nth) {
                    const bool pre = s == s0 + spread && st.d.z >= 0;
                    if (res_skip(sb, rc, s)) {
                        if (pre && st.e) cp_async_wait();   // staged copies complete before the pool is reused
                        continue;
                    }
                    const int4 d = pre ? st.d : R.slot_desc[s];
                    const float2 im = pre ? st.im : R.slot_im[s];
                    PoolSlot ps;
                    if (pre && st.e) { ps.e = st.e; ps.j0 = 0; }
                    else ps = pool_take(pp, R, kind, d.z);
                    V l0, a0, l1, a1;
                    gload(w, d.x, l0, a0);
                    gload(w, d.y, l1, a1);
                    Resid res;
                    if (rc.on) solve_manifold<true>(w, R, s, d.z, kind, l0, a0, l1, a1, im.x, im.y, res, ps);
                    else solve_manifold<false>(w, R, s, d.z, kind, l0, a0, l1, a1, im.x, im.y, res, ps);
                    res_keep(sb, rc, kind, s, res);
                    if (im.x != 0.0f) gstore(w, d.x, l0, a0);
                    if (im.y != 0.0f) gstore(w, d.y, l1, a1);
                }
                st.d = dn;
                st.im = imn;
                st.e = dn.z >= 0 ? pool_copy(pool(step + 1), R, kind, dn.z, 0) : nullptr;
                grid_barrier(w.ctr, nb, barK);
                ++step;
            }
        }
        ++it;
        if (it >= maxIt) break;
        if (byRes && it > 0 && contacts) {
            // island residuals of this iteration; ctr[C_RES0 + it % 3] counts islands still
            // above the tolerance, the next slot is cleared (last read two iterations ago)
            const int flag = C_RES0 + it % 3;
            if (tid == 0) w.ctr[C_RES0 + (it + 1) % 3] = 0;
            island_residuals(w, sb, flag, it);
            grid_barrier(w.ctr, nb, barK);
            if (__ldcg(&w.ctr[flag]) == 0) break;
            rc.skipConv = true;
        }
    }
    if (tid == 0 && it > 0) atomicMax(&w.ctr[C_PGS_ITERS], it);
    if (byRes && contacts) {   // per-island statistics: islConv holds the iteration an island converged at
        const int nChunks = *sb.nIslChunks;
        for (int ch = tid; ch < nChunks; ch += nth) {
            const int2 cd = sb.islChunk[ch];
            if (cd.y != 0) continue;
            const int c = __ldcg(&sb.islConv[cd.x]);
            atomicAdd(&w.ctr[C_ISL_N], 1);
            if (c > 0) atomicAdd(&w.ctr[C_ISL_CONV], 1);
            atomicAdd(&w.ctr[C_ISL_ITERS], c > 0 ? c : it);
        }
    }
    for (int s = tid; s < nSlots; s += nth) writeback_slot(P, R, s);
}

// Island index of every solve slot and the slots grouped by island (residual mode).
__global__ void k_isl_count(DevWorld w, DevRows R, SolverBuffers sb) {
    int nSlots = *sb.nCand;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nSlots) return;
    int4 d = R.slot_desc[s];
    // world scope: every slot in one group (index 0), tested against one residual
    int isl = w.resScope ? 0 : (w.island[d.x] >= 0 ? w.island[d.x] : w.island[d.y]);
    sb.slotIsl[s] = isl;
    atomicAdd(&sb.islCount[isl], 1);
}
__global__ void k_isl_scatter(SolverBuffers sb, int nBodies) {
    int nSlots = *sb.nCand;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nSlots) {
        int isl = sb.slotIsl[s];
        sb.islList[sb.islStart[isl] + atomicAdd(&sb.islFill[isl], 1)] = s;
    }
    if (s < nBodies) sb.segFlag[s] = (sb.islCount[s] + ISL_CHUNK - 1) / ISL_CHUNK;   // chunks of island s
}
__global__ void k_isl_segments(SolverBuffers sb, int nBodies) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nBodies) return;
    int nch = (sb.islCount[i] + ISL_CHUNK - 1) / ISL_CHUNK;
    for (int c = 0; c < nch; c++) sb.islChunk[sb.segIdx[i] + c] = make_int2(i, c);
}

// ---- learned warm start and contact samples ------------------------------------------------
// Features of contact point q = slot * 4 + j (24 floats), from the rows just set up and the body
// state before the solve: normal (3), distance (1), relative velocity at the contact (3),
// relative angular velocity (3), inverse masses (2), inverse-inertia-projected normals of
// both bodies (6), the point's previous applied impulse and lateral impulses (3), friction,
// restitution (2), lifetime (1).
JBD void contact_features(const DevWorld& w, const DevPairs& P, const DevRows& R, int ni, float* f) {
    const int s = R.pt_key[ni] >> 2, j = R.pt_key[ni] & 3;
    const int p = R.slot_pair[s], k = p * 4 + j;
    const int4 d = R.slot_desc[s];
    const float2 im = R.slot_im[s];
    float4 nn = R.n_nrm[ni], aA = R.n_angA[ni], aB = R.n_angB[ni];
    float4 wa = P.wA[k], wb = P.wB[k], pa = P.pA[k], pb = P.pB[k], nr = P.nrm[k], ii = P.imp[k];
    V com0 = mk(w.xr0[d.x].w, w.xr1[d.x].w, w.xr2[d.x].w), com1 = mk(w.xr0[d.y].w, w.xr1[d.y].w, w.xr2[d.y].w);
    V l0 = mk4(w.linvel[d.x]), a0 = mk4(w.angvel[d.x]), l1 = mk4(w.linvel[d.y]), a1 = mk4(w.angvel[d.y]);
    V rp1 = sub(mk(wa.x, wa.y, wa.z), com0), rp2 = sub(mk(wb.x, wb.y, wb.z), com1);
    V vel = sub(add(crs(a0, rp1), l0), add(crs(a1, rp2), l1));
    V dw = sub(a0, a1);
    f[0] = nn.x; f[1] = nn.y; f[2] = nn.z;
    f[3] = pa.w;
    f[4] = vel.x; f[5] = vel.y; f[6] = vel.z;
    f[7] = dw.x; f[8] = dw.y; f[9] = dw.z;
    f[10] = im.x; f[11] = im.y;
    f[12] = aA.x; f[13] = aA.y; f[14] = aA.z;
    f[15] = aB.x; f[16] = aB.y; f[17] = aB.z;
    f[18] = nr.w; f[19] = ii.x; f[20] = ii.y;
    f[21] = aA.w; f[22] = wb.w;
    f[23] = (float)__float_as_int(pb.w);
}

__global__ void k_contact_features(DevWorld w, DevPairs P, DevRows R, const int* nPtsPtr, float* X) {
    const int nq = *nPtsPtr;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        float f[MLP_IN];
        contact_features(w, P, R, q, f);
        for (int e = 0; e < MLP_IN; e++) X[(size_t)q * MLP_IN + e] = f[e];
    }
}

// Targets of points whose island did not reach the residual (residual mode) are NaN: they are
// not converged impulses, and the sample export leaves them out.
__global__ void k_contact_targets(DevWorld w, DevRows R, SolverBuffers sb, float* T, int allPoints) {
    const int nq = *R.nPts;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        if (!allPoints && w.resTol > 0.0f && __ldcg(&sb.islConv[sb.slotIsl[R.pt_key[q] >> 2]]) == 0) {
            T[(size_t)q * 3 + 0] = T[(size_t)q * 3 + 1] = T[(size_t)q * 3 + 2] = __int_as_float(0x7fc00000);
            continue;
        }
        T[(size_t)q * 3 + 0] = R.n_angB[q].w;
        T[(size_t)q * 3 + 1] = R.f_rp1[q * 2].w;
        T[(size_t)q * 3 + 2] = R.f_rp1[q * 2 + 1].w;
    }
}

// Warm-start impulses predicted by the MLP for 64 contact points per tile.  The network's three
// outputs o give y = MLP_REL sinh(o), relative to the point's last normal impulse b (feature 18)
// and an impulse scale u = unit / (invMass0 + invMass1): normal = max(0, b + y0 (b + u)),
// friction k = y(1+k) mu (b + u) clamped to the cone of that normal impulse.  They replace warmstartingFactor x last step's
// impulses before the PGS warm-start phase.
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_warmstart(DevWorld w, DevPairs P, DevRows R, MlpDev M) {
    extern __shared__ __align__(16) unsigned char mlpSmem[];
    MlpSmem& S = *reinterpret_cast<MlpSmem*>(mlpSmem);
    const int nq = *R.nPts;
    mlp_load_weights(S, M);
    for (int first = blockIdx.x * MLP_TILE; first < nq; first += gridDim.x * MLP_TILE) {
        if (threadIdx.x < MLP_TILE) {
            const int q = first + threadIdx.x;
            float f[MLP_IN];
            bool on = q < nq;
            if (on) contact_features(w, P, R, q, f);
            for (int e = 0; e < MLP_INP; e++) {
                float v = (on && e < MLP_IN) ? mlp_norm_in(M.norm, e, f[e]) : 0.0f;
                S.x[threadIdx.x][e] = __float2bfloat16_rn(v);
            }
        }
        __syncthreads();
        mlp_forward(S, M);
        if (threadIdx.x < MLP_TILE) {
            const int q = first + threadIdx.x;
            if (q < nq) {
                const int key = R.pt_key[q];
                float y[MLP_OUT];
                for (int o = 0; o < MLP_OUT; o++)
                    y[o] = MLP_REL * sinhf(S.y[threadIdx.x][o] * M.norm[2 * MLP_IN + MLP_OUT + o] + M.norm[2 * MLP_IN + o]);
                const float2 im = R.slot_im[key >> 2];
                const float base = fmaxf(P.nrm[R.slot_pair[key >> 2] * 4 + (key & 3)].w, 0.0f);
                const float unit = M.norm[MLP_NORM_UNIT] / fmaxf(im.x + im.y, 1e-6f);
                const float mu = R.n_angA[q].w;
                float ln = base + y[0] * (base + unit);
                ln = ln > 0.0f ? ln : 0.0f;
                float lim = ln * mu;
                float4 b = R.n_angB[q];
                b.w = ln;
                R.n_angB[q] = b;
                for (int f2 = 0; f2 < 2; f2++) {
                    float v = y[1 + f2] * mu * (base + unit);
                    v = v > lim ? lim : (v < -lim ? -lim : v);
                    float4 r = R.f_rp1[q * 2 + f2];
                    r.w = v;
                    R.f_rp1[q * 2 + f2] = r;
                }
            }
        }
        __syncthreads();
    }
}

// ---- host side ------------------------------------------------------------------------------
template <class T> static cudaError_t salloc(T** p, size_t n) {
    return cudaMalloc((void**)p, sizeof(T) * (n ? n : 1));
}
template <class T> static void sfree(T*& p) { if (p) cudaFree((void*)p); p = nullptr; }

static size_t pgs_smem(const SolverBuffers& sb) {
    return (sb.partSmem ? (size_t)sb.smemCap * 32 : 0) + (size_t)3 * sb.poolPts * POOL_F4 * 16;
}
static size_t colour_smem(const SolverBuffers& sb) { return (size_t)sb.partMax * (sizeof(unsigned long long) + sizeof(int)); }

int solver_configure(SolverBuffers& sb, int nFinite, const std::vector<int>& worldCounts, int sms, int rangeParts,
                     int threads, int smemBodies) {
    sb.threads = threads;
    int maxWorld = 0;
    for (int c : worldCounts) maxWorld = std::max(maxWorld, c);
    std::vector<int> start;
    int parts;
    if (rangeParts <= 0 && !worldCounts.empty() && maxWorld <= PART_MAX_BODIES) {
        sb.worldParts = 1;
        parts = (int)worldCounts.size();
        start.resize(parts + 1);
        start[0] = 0;
        for (int p = 0; p < parts; p++) start[p + 1] = start[p] + worldCounts[p];
    } else {
        sb.worldParts = 0;
        const int minParts = (nFinite + PART_MAX_BODIES - 1) / PART_MAX_BODIES;
        parts = std::max(rangeParts > 0 ? rangeParts : 2 * sms, minParts);
        parts = std::max(1, std::min(parts, std::max(nFinite, 1)));
        start.resize(parts + 1);
        for (int p = 0; p <= parts; p++) start[p] = (int)(((long long)p * nFinite + parts - 1) / parts);
    }
    int partMax = 1;
    for (int p = 0; p < parts; p++) partMax = std::max(partMax, start[p + 1] - start[p]);
    if (parts > sb.partsCap) {
        sfree(sb.bucketCount); sfree(sb.bucketFill); sfree(sb.bucketStart);
        sfree(sb.lcCount); sfree(sb.lcFill); sfree(sb.lcStart); sfree(sb.nLocal); sfree(sb.partStart); sfree(sb.partOrder);
        size_t lc = (size_t)parts * (MAX_LOCAL + 1);
        if (salloc(&sb.bucketCount, parts + 2) || salloc(&sb.bucketFill, parts + 2) || salloc(&sb.bucketStart, parts + 2) ||
            salloc(&sb.lcCount, lc) || salloc(&sb.lcFill, lc) || salloc(&sb.lcStart, lc) || salloc(&sb.nLocal, parts) ||
            salloc(&sb.partStart, parts + 1) || salloc(&sb.partOrder, parts)) {
            sb.partsCap = 0;
            return JBGPU_ERR_CUDA;
        }
        sb.partsCap = parts;
    }
    std::vector<int> order(parts);
    for (int p = 0; p < parts; p++) order[p] = p;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return start[a + 1] - start[a] > start[b + 1] - start[b]; });
    if (cudaMemcpy(sb.partStart, start.data(), sizeof(int) * (parts + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(sb.partOrder, order.data(), sizeof(int) * parts, cudaMemcpyHostToDevice) != cudaSuccess)
        return JBGPU_ERR_CUDA;
    sb.nFinite = nFinite;
    sb.nParts = parts;
    sb.partMax = partMax;
    sb.smemCap = std::min(partMax, smemBodies > 0 ? smemBodies : PART_MAX_BODIES);
    sb.partSmem = (sb.smemCap < 0xffff && (size_t)sb.smemCap * 32 <= 96 * 1024) ? 1 : 0;
    // one k_pgs attribute value for every world of the process (a smaller value set by another
    // world would invalidate this world's occupancy)
    int dev = 0, smemBlock = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smemBlock, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncSetAttribute(k_pgs, cudaFuncAttributeMaxDynamicSharedMemorySize, smemBlock - 1024) != cudaSuccess)
        return JBGPU_ERR_CUDA;
    // point pools: half a block's threads in entries (a quarter with world parts, whose blocks
    // stage nothing ahead and keep more of the SM as L1), fewer or none if they would cost
    // occupancy
    int perPgs = 0, perColour = 0, perBare = 0;
    sb.poolPts = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perBare, k_pgs, threads, pgs_smem(sb)) != cudaSuccess)
        return JBGPU_ERR_CUDA;
    for (int pts = sb.worldParts ? threads / 4 : threads / 2; pts >= 16; pts /= 2) {
        sb.poolPts = pts;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perPgs, k_pgs, threads, pgs_smem(sb)) != cudaSuccess)
            return JBGPU_ERR_CUDA;
        if (perPgs >= perBare) break;
        sb.poolPts = 0;
    }
    size_t smem = pgs_smem(sb);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perPgs, k_pgs, threads, smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perColour, k_colour, threads, colour_smem(sb)) != cudaSuccess ||
        perPgs < 1 || perColour < 1)
        return JBGPU_ERR_CUDA;
    sb.gridPgs = std::min(parts, perPgs * sms);
    sb.gridColour = std::min(parts, perColour * sms);
    return JBGPU_OK;
}

void solver_free(SolverBuffers& sb) {
    sfree(sb.bucketCount); sfree(sb.bucketFill); sfree(sb.bucketStart);
    sfree(sb.lcCount); sfree(sb.lcFill); sfree(sb.lcStart); sfree(sb.nLocal); sfree(sb.partStart); sfree(sb.partOrder);
    sfree(sb.orderFallback);
    sb.partsCap = 0;
}

size_t mlp_smem_bytes();   // mlp.cu

int solver_learn_configure() {
    return cudaFuncSetAttribute(k_mlp_warmstart, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem_bytes()) ==
                   cudaSuccess ? 0 : 1;
}

void solve_launch(const DevWorld& w, DevPairs& P, int nPairs, DevRows& R, SolverBuffers& sb, float dt, cudaStream_t s,
                  const Prof* prof) {
    solve_launch_learn(w, P, nPairs, R, sb, dt, s, prof, SolverLearn());
}

void solve_launch_learn(const DevWorld& w, DevPairs& P, int nPairs, DevRows& R, SolverBuffers& sb, float dt,
                        cudaStream_t s, const Prof* prof, const SolverLearn& learn) {
    if (prof) prof->mark(PH_COLOUR, 0, s);
    if (nPairs <= 0 || sb.nFinite <= 0 || sb.nParts <= 0) {
        cudaMemsetAsync(sb.nColours, 0, sizeof(int), s);
        cudaMemsetAsync(sb.nCand, 0, sizeof(int), s);
        if (prof) { prof->mark(PH_COLOUR, 1, s); prof->mark(PH_SETUP, 0, s); }
        const bool joints = sb.J.n > 0 && sb.nFinite > 0 && sb.nParts > 0;
        if (joints) { k_joint_setup<<<gridn(sb.J.n, 128), 128, 0, s>>>(w, sb); note_launch(); }
        if (prof) { prof->mark(PH_SETUP, 1, s); prof->mark(PH_PGS, 0, s); }
        if (joints) {   // no contact manifold: the joints alone
            cudaMemsetAsync(w.ctr + C_BAR_COUNT, 0, sizeof(int), s);
            cudaMemsetAsync(w.ctr + C_PGS_ITERS, 0, sizeof(int), s);
            DevWorld wc = w;
            DevPairs pc = P;
            DevRows rc = R;
            SolverBuffers sc = sb;
            float dtc = dt;
            void* args[] = {&wc, &pc, &rc, &sc, &dtc};
            cudaLaunchCooperativeKernel((void*)k_pgs, sb.gridPgs, sb.threads, args, pgs_smem(sb), s); note_launch();
        }
        if (prof) prof->mark(PH_PGS, 1, s);
        return;
    }
    const int parts = sb.nParts;
    cudaMemsetAsync(sb.claim, 0xff, sizeof(unsigned long long) * w.nBodies, s);
    cudaMemsetAsync(sb.taken, 0xff, sizeof(int) * w.nBodies, s);
    cudaMemsetAsync(sb.posOf, 0xff, sizeof(int) * w.nBodies, s);
    cudaMemsetAsync(sb.bucketCount, 0, sizeof(int) * (parts + 2), s);
    cudaMemsetAsync(sb.bucketFill, 0, sizeof(int) * (parts + 2), s);
    cudaMemsetAsync(sb.lcFill, 0, sizeof(int) * parts * (MAX_LOCAL + 1), s);
    cudaMemsetAsync(sb.colourFill, 0, sizeof(int) * (MAX_COLOURS + 1), s);
    cudaMemsetAsync(w.ctr + C_BAR_COUNT, 0, sizeof(int), s);
    cudaMemsetAsync(w.ctr + C_PGS_ITERS, 0, sizeof(int), s);
    cudaMemsetAsync(w.ctr + C_ISL_N, 0, sizeof(int) * 5, s);   // island statistics, part counters
    k_posof<<<gridn(sb.nFinite, 256), 256, 0, s>>>(sb); note_launch();
    k_classify<<<gridn(nPairs, 256), 256, 0, s>>>(w, P, sb); note_launch();
    exclusive_scan(sb.bucketCount, sb.bucketStart, nullptr, parts + 2, sb.scanScratch, s);
    k_bucket_scatter<<<gridn(nPairs, 256), 256, 0, s>>>(sb); note_launch();
    {
        DevWorld wc = w;
        DevPairs pc = P;
        SolverBuffers sc = sb;
        void* args[] = {&wc, &pc, &sc};
        cudaLaunchCooperativeKernel((void*)k_colour, sb.gridColour, sb.threads, args, colour_smem(sb), s); note_launch();
    }
    k_slots<<<gridn(nPairs, 256), 256, 0, s>>>(w, P, sb, R); note_launch();
    if (w.resTol > 0.0f) {        // residual mode: slots grouped by island
        const int n = w.nBodies;
        cudaMemsetAsync(sb.islCount, 0, sizeof(int) * (n + 1), s);
        cudaMemsetAsync(sb.islFill, 0, sizeof(int) * (n + 1), s);
        cudaMemsetAsync(sb.islConv, 0, sizeof(int) * n, s);
        cudaMemsetAsync(sb.islAcc, 0, sizeof(int) * 2 * n, s);
        cudaMemsetAsync(sb.islDone, 0, sizeof(int) * n, s);
        cudaMemsetAsync(sb.resTrace, 0, sizeof(unsigned) * 2 * JBGPU_RESIDUAL_TRACE_MAX, s);
        k_isl_count<<<gridn(nPairs, 256), 256, 0, s>>>(w, R, sb); note_launch();
        exclusive_scan(sb.islCount, sb.islStart, nullptr, n + 1, sb.islScratch, s);
        k_isl_scatter<<<gridn(std::max(nPairs, n), 256), 256, 0, s>>>(sb, n); note_launch();
        exclusive_scan(sb.segFlag, sb.segIdx, sb.nIslChunks, n, sb.islScratch, s);
        k_isl_segments<<<gridn(n, 256), 256, 0, s>>>(sb, n); note_launch();
    }
    if (prof) { prof->mark(PH_COLOUR, 1, s); prof->mark(PH_SETUP, 0, s); }
    k_point_masks<<<gridn(nPairs, 256), 256, 0, s>>>(P, R, sb.nCand, nPairs); note_launch();
    exclusive_scan(R.slot_pt0, R.slot_pt0, R.nPts, nPairs, sb.scanScratch, s);
    k_point_rows<<<gridn(nPairs, 256), 256, 0, s>>>(R, sb.nCand); note_launch();
    k_setup<<<gridn(nPairs, 128), 128, 0, s>>>(w, P, R, sb.nCand, dt); note_launch();
    if (learn.sampleX) {
        k_contact_features<<<std::min(gridn(nPairs * 4, 256), 4096), 256, 0, s>>>(w, P, R, R.nPts, learn.sampleX);
        note_launch();
    }
    if (learn.mlp) {
        int tiles = std::min(gridn(nPairs * 4, MLP_TILE), 2048);
        k_mlp_warmstart<<<tiles, MLP_THREADS, mlp_smem_bytes(), s>>>(w, P, R, *learn.mlp);
        note_launch();
    }
    if (sb.J.n > 0) { k_joint_setup<<<gridn(sb.J.n, 128), 128, 0, s>>>(w, sb); note_launch(); }
    if (prof) { prof->mark(PH_SETUP, 1, s); prof->mark(PH_PGS, 0, s); }
    cudaMemsetAsync(w.ctr + C_BAR_COUNT, 0, sizeof(int), s);
    {
        DevWorld wc = w;
        DevPairs pc = P;
        DevRows rc = R;
        SolverBuffers sc = sb;
        float dtc = dt;
        void* args[] = {&wc, &pc, &rc, &sc, &dtc};
        cudaLaunchCooperativeKernel((void*)k_pgs, sb.gridPgs, sb.threads, args, pgs_smem(sb), s); note_launch();
    }
    if (prof) prof->mark(PH_PGS, 1, s);
    if (learn.sampleT) {
        k_contact_targets<<<std::min(gridn(nPairs * 4, 256), 4096), 256, 0, s>>>(w, R, sb, learn.sampleT,
                                                                                 learn.allPoints);
        note_launch();
    }
}

}  // namespace jbg
