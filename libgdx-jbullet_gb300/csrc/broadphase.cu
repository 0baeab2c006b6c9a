// Broadphase: the overlapping-pair set of the reference's DbvtBroadphase, rebuilt each step.
//
// The reference keeps an incremental dynamic AABB tree and, after collide(), its pair cache
// holds exactly the filter-passing pairs whose proxy aabbs intersect inclusively
// (collision/broadphase/DbvtBroadphase.java:89-150, DbvtTreeCollider.java:36-51,
// DbvtAabbMm.java:209-212, HashedOverlappingPairCache.java:179-188).  Here:
//   1. 30-bit Morton codes of finite proxy aabb centres, world index in the high key bits;
//   2. stable radix sort; 3. Karras radix tree over the sorted leaves (one root per world);
//   4. bottom-up refit; 5. a counting traversal (pair owner = the lower body index, or the
//   finite body of a pair with a static plane), exclusive scan -> per-owner CSR;
//   6. a filling traversal, per-owner partner sort -> keys sorted ascending;
//   7. persistence: each new key is looked up among last step's sorted keys and its
//   manifold (the reference's algorithm lifetime, HashedOverlappingPairCache.java:222-228) is
//   carried over.
// Static planes (infinite aabb, StaticPlaneShape.java:124-128) stay out of the tree; each
// finite body tests the planes of its world directly.
#include <utility>

#include "broadphase.cuh"
#include "dispatch.cuh"
#include "prims.cuh"

namespace jbg {
using namespace jbd;

__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Scene bounds of finite aabb centres (ordered-int atomics).
__global__ void k_bounds(DevWorld w, unsigned* bnd) {
    __shared__ unsigned s[6];
    if (threadIdx.x < 6) s[threadIdx.x] = (threadIdx.x < 3) ? 0xffffffffu : 0u;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < w.nBodies && !(w.flags[i] & CF_LISTED)) {
        float4 a = w.amin[i], b = w.amax[i];
        float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
        for (int k = 0; k < 3; k++) {
            atomicMin(&s[k], f2ord(c[k]));
            atomicMax(&s[3 + k], f2ord(c[k]));
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) atomicMin(&bnd[threadIdx.x], s[threadIdx.x]);
    else if (threadIdx.x < 6) atomicMax(&bnd[threadIdx.x], s[threadIdx.x]);
}

__device__ __forceinline__ unsigned expand_bits(unsigned v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// key = world << 32 | morton30 for finite bodies; planes get the all-ones key (sorted last).
__global__ void k_morton(DevWorld w, const unsigned* bnd, uint64_t* keys, int* vals) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies) return;
    vals[i] = i;
    if (w.flags[i] & CF_LISTED) { keys[i] = ~0ull; return; }
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) { lo[k] = ord2f(bnd[k]); hi[k] = ord2f(bnd[3 + k]); }
    float4 a = w.amin[i], b = w.amax[i];
    float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    unsigned q[3];
    for (int k = 0; k < 3; k++) {
        float ext = hi[k] - lo[k];
        float t = ext > 0.0f ? (c[k] - lo[k]) / ext : 0.5f;
        t = fminf(fmaxf(t, 0.0f), 1.0f);
        q[k] = min((unsigned)(t * 1024.0f), 1023u);
    }
    unsigned m = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    keys[i] = ((uint64_t)(unsigned)w.world[i] << 32) | m;
}

__device__ __forceinline__ int delta(const uint64_t* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = k[i], b = k[j];
    if (a == b) return 64 + __clz(i ^ j);
    return __clzll(a ^ b);
}

// World leaf ranges in the sorted leaf order; single-leaf worlds get the leaf as root.
__global__ void k_world_ranges(const uint64_t* keys, int nf, int* wstart, int* wend, int* wroot) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    int wi = (int)(keys[i] >> 32);
    if (i == 0 || (int)(keys[i - 1] >> 32) != wi) wstart[wi] = i;
    if (i == nf - 1 || (int)(keys[i + 1] >> 32) != wi) {
        wend[wi] = i + 1;
        int s = (i == 0 || (int)(keys[i - 1] >> 32) != wi) ? i : -1;
        if (s == i) wroot[wi] = LEAF_FLAG | i;
    }
}

// Karras 2012 radix-tree construction over nf sorted leaves.
__global__ void k_karras(const uint64_t* keys, int nf, Bvh t, const int* wstart, const int* wend, int* wroot) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf - 1) return;
    int d = (delta(keys, nf, i, i + 1) - delta(keys, nf, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, nf, i, i - d);
    int lmax = 2;
    while (delta(keys, nf, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int s = lmax >> 1; s >= 1; s >>= 1)
        if (delta(keys, nf, i, i + (l + s) * d) > dmin) l += s;
    int j = i + l * d;
    int dnode = delta(keys, nf, i, j);
    int s = 0, tt = l;
    do {
        tt = (tt + 1) >> 1;
        if (delta(keys, nf, i, i + (s + tt) * d) > dnode) s += tt;
    } while (tt > 1);
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    int left = (lo == gamma) ? (LEAF_FLAG | gamma) : gamma;
    int right = (hi == gamma + 1) ? (LEAF_FLAG | (gamma + 1)) : (gamma + 1);
    t.left[i] = left;
    t.right[i] = right;
    t.lo[i] = lo;
    t.hi[i] = hi;
    if (left & LEAF_FLAG) t.leafParent[gamma] = i; else t.parent[gamma] = i;
    if (right & LEAF_FLAG) t.leafParent[gamma + 1] = i; else t.parent[gamma + 1] = i;
    int wi = (int)(keys[lo] >> 32);
    if (wstart[wi] == lo && wend[wi] == hi + 1) wroot[wi] = i;
}

// Bottom-up refit into the parents' child records: a leaf writes its box into its parent's
// record; the second child to arrive at a node merges the node's two child boxes and writes the
// union into the node's slot in its own parent (roots have parent -1).
__global__ void k_refit(DevWorld w, const int* sortedBody, int nf, Bvh t) {
    int leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= nf) return;
    const int b = sortedBody[leaf];
    float4 mn = w.amin[b], mx = w.amax[b];
    int child = LEAF_FLAG | leaf, last = leaf;
    int node = t.leafParent[leaf];
    while (node >= 0) {
        const int side = t.left[node] == child ? 0 : 2;
        __stcg(&t.node[4 * node + side], make_float4(mn.x, mn.y, mn.z, __int_as_float(child)));
        __stcg(&t.node[4 * node + side + 1], make_float4(mx.x, mx.y, mx.z, __int_as_float(last)));
        // release: this child's record; acquire: the sibling's (the second arrival goes on)
        int prev;
        asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(prev) : "l"(t.visit + node) : "memory");
        if (prev == 0) return;
        const float4 l0 = __ldcg(&t.node[4 * node]), l1 = __ldcg(&t.node[4 * node + 1]);
        const float4 r0 = __ldcg(&t.node[4 * node + 2]), r1 = __ldcg(&t.node[4 * node + 3]);
        mn = make_float4(fminf(l0.x, r0.x), fminf(l0.y, r0.y), fminf(l0.z, r0.z), 0.0f);
        mx = make_float4(fmaxf(l1.x, r1.x), fmaxf(l1.y, r1.y), fmaxf(l1.z, r1.z), 0.0f);
        child = node;
        last = t.hi[node];
        node = t.parent[node];
    }
}

__device__ __forceinline__ bool ovl(float4 a0, float4 a1, float4 b0, float4 b1) {
    return (a0.x <= b1.x) && (a1.x >= b0.x) && (a0.y <= b1.y) && (a1.y >= b0.y) && (a0.z <= b1.z) && (a1.z >= b0.z);
}
__device__ __forceinline__ bool filt(const DevWorld& w, int a, int b) {
    return (w.group[a] & w.mask[b]) != 0 && (w.group[b] & w.mask[a]) != 0;
}

constexpr int STACK = 96;

// One leaf's traversal: pairs (s, t) with t > s in sorted order.  FILL == false counts
// pairs per owner and keeps up to TRAV_CACHE of leaf s's partners; FILL == true writes partners
// into the owner's CSR segment, from that cache when it holds all of them, else by traversing
// again.
template <bool FILL>
__global__ void k_traverse(DevWorld w, const int* sortedBody, int nf, Bvh t, const int* wroot, int* cnt, const int* off,
                           int* cursor, int* partners, int capacity, int* tcount, int* tcache) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    int bi = sortedBody[s];
    auto emit = [&](int bj) {
        int owner = bi < bj ? bi : bj, partner = bi < bj ? bj : bi;
        const int subs = w.hasCompound ? pair_subs(w.sh, w.shape[owner], w.shape[partner]) : 1;
        if (!FILL) {
            atomicAdd(&cnt[owner], subs);
        } else {
            int pos = off[owner] + atomicAdd(&cursor[owner], subs);
            for (int k = 0; k < subs; k++)
                if (pos + k < capacity) partners[pos + k] = partner | (k << 24);
        }
    };
    if (FILL) {
        const int found = tcount[s];
        if (found <= TRAV_CACHE) {
            for (int i = 0; i < found; i++) emit(sortedBody[tcache[(size_t)s * TRAV_CACHE + i]]);
            return;
        }
    }
    int root = wroot[w.world[bi]];
    if (root & LEAF_FLAG) {   // single-leaf world
        if (!FILL) tcount[s] = 0;
        return;
    }
    float4 a0 = w.amin[bi], a1 = w.amax[bi];
    int found = 0;
    int stack[STACK];
    int sp = 0;
    stack[sp++] = root;
    while (sp > 0) {
        const float4* nd = t.node + 4 * stack[--sp];
        const float4 rec[4] = {nd[0], nd[1], nd[2], nd[3]};
        for (int c = 0; c < 2; c++) {
            const float4 mn = rec[2 * c], mx = rec[2 * c + 1];
            if (__float_as_int(mx.w) <= s) continue;   // the child's leaves all precede s
            if (!ovl(a0, a1, mn, mx)) continue;
            const int x = __float_as_int(mn.w);
            if (x & LEAF_FLAG) {
                const int tl = x & ~LEAF_FLAG;
                const int bj = sortedBody[tl];
                if (!filt(w, bi, bj)) continue;
                emit(bj);
                if (!FILL && found < TRAV_CACHE) tcache[(size_t)s * TRAV_CACHE + found] = tl;
                ++found;
            } else {
                if (sp < STACK) stack[sp++] = x;
                else atomicOr(&w.ctr[C_STATUS], ST_CAPACITY);
            }
        }
    }
    if (!FILL) tcount[s] = found;
}

// Pairs of each body in the tree with the listed bodies (static planes, triangle meshes) of its
// world, owned by the former.
// The counting pass also sums, into candBound, the triangle candidates the concave pass will
// list for the body's mesh pairs (an upper bound: pairs whose bodies are both inactive list none).
template <bool FILL>
__global__ void k_plane_pairs(DevWorld w, const int* planeList, const int* planeStart, int* cnt, const int* off,
                              int* cursor, int* partners, int capacity, int* candBound) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nBodies || (w.flags[i] & CF_LISTED)) return;
    int wi = w.world[i];
    float4 a0 = w.amin[i], a1 = w.amax[i];
    for (int k = planeStart[wi]; k < planeStart[wi + 1]; k++) {
        int p = planeList[k];
        if (!ovl(a0, a1, w.amin[p], w.amax[p]) || !filt(w, i, p)) continue;
        const int subs = w.hasCompound ? pair_subs(w.sh, w.shape[i], w.shape[p]) : 1;
        if (!FILL && candBound) {
            const int c = mesh_candidates(w, i, p);
            if (c) atomicAdd(candBound, c);
        }
        if (!FILL) atomicAdd(&cnt[i], subs);
        else {
            int pos = off[i] + atomicAdd(&cursor[i], subs);
            for (int k = 0; k < subs; k++)
                if (pos + k < capacity) partners[pos + k] = p | (k << 24);
        }
    }
}

// Ascending sort of c words in place: in registers up to 32, else a Shell sort in memory.
JBD void sort_words(unsigned* p, int c) {
    if (c <= 32) {
        unsigned v[32];
        for (int k = 0; k < c; k++) v[k] = p[k];
        for (int k = 1; k < c; k++) {
            unsigned x = v[k];
            int j = k - 1;
            while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; j--; }
            v[j + 1] = x;
        }
        for (int k = 0; k < c; k++) p[k] = v[k];
        return;
    }
    for (int gap = c / 2; gap > 0; gap /= 2)
        for (int k = gap; k < c; k++) {
            unsigned x = p[k];
            int j = k;
            while (j >= gap && p[j - gap] > x) { p[j] = p[j - gap]; j -= gap; }
            p[j] = x;
        }
}

// Sort each owner's partner words (sub << 24 | partner, compared unsigned) ascending and emit the
// canonical keys.  With compounds a partner's child combinations are written together, so the
// owner's distinct partners (the words with sub 0) are sorted alone and the keys generated sub
// by sub - the same ascending order without sorting every combination.
__global__ void k_segment_sort(DevWorld w, int n, const int* off, const int* cnt, int* partners, uint64_t* keys,
                               int capacity) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int o = off[i], c = cnt[i];
    if (o + c > capacity) return;
    unsigned* p = (unsigned*)partners + o;
    if (w.hasCompound) {
        int np = 0;
        for (int k = 0; k < c; k++)
            if ((p[k] >> 24) == 0) p[np++] = p[k];   // in place: np <= k
        sort_words(p, np);
        const uint64_t hi = (uint64_t)(unsigned)i << 32;
        int at = 0, more = 1;
        for (unsigned sub = 0; more && at < c; sub++) {
            more = 0;
            for (int k = 0; k < np; k++) {
                const int subs = pair_subs(w.sh, w.shape[i], w.shape[p[k]]);
                if ((int)sub < subs) {
                    keys[o + at++] = hi | (sub << 24) | p[k];
                    more |= (int)sub + 1 < subs;
                }
            }
        }
        return;
    }
    if (c <= 32) {
        unsigned v[32];
        for (int k = 0; k < c; k++) v[k] = p[k];
        for (int k = 1; k < c; k++) {
            unsigned x = v[k];
            int j = k - 1;
            while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; j--; }
            v[j + 1] = x;
        }
        for (int k = 0; k < c; k++) keys[o + k] = ((uint64_t)(unsigned)i << 32) | v[k];
    } else {
        for (int gap = c / 2; gap > 0; gap /= 2)          // Shell sort for rare crowded owners
            for (int k = gap; k < c; k++) {
                unsigned x = p[k];
                int j = k;
                while (j >= gap && p[j - gap] > x) { p[j] = p[j - gap]; j -= gap; }
                p[j] = x;
            }
        for (int k = 0; k < c; k++) keys[o + k] = ((uint64_t)(unsigned)i << 32) | p[k];
    }
}

// The same for worlds without compounds, in two passes.  A thread per owner sorts a segment of up
// to SEG_REG partner words in registers (a bitonic network over 8, padding words 0xffffffff
// sorting last) and lists the owners of longer segments; then a warp per listed owner sorts up
// to 32 words across the lanes by a bitonic network, a crowded segment in place by one lane.
constexpr int SEG_REG = 8;
__global__ void k_segment_sort_short(int n, const int* off, const int* cnt, const int* partners, uint64_t* keys,
                                     int capacity, int* longList, int* longCount) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;   // the grid covers whole warps
    int o = 0, c = 0;
    if (i < n) {
        o = off[i];
        c = cnt[i];
        if (o + c > capacity) c = 0;
    }
    if (c > 0 && c <= SEG_REG) {
        const unsigned* p = (const unsigned*)partners + o;
        unsigned r[SEG_REG];
#pragma unroll
        for (int k = 0; k < SEG_REG; k++) r[k] = k < c ? p[k] : 0xffffffffu;
#pragma unroll
        for (int k = 2; k <= SEG_REG; k <<= 1)
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
                for (int a = 0; a < SEG_REG; a++) {
                    const int b = a ^ j;
                    if (b > a) {
                        const unsigned x = r[a], y = r[b];
                        if ((x > y) == ((a & k) == 0)) { r[a] = y; r[b] = x; }
                    }
                }
        const uint64_t hi = (uint64_t)(unsigned)i << 32;
#pragma unroll
        for (int k = 0; k < SEG_REG; k++)
            if (k < c) keys[o + k] = hi | r[k];
    }
    const bool lng = c > SEG_REG;
    const unsigned m = __ballot_sync(0xffffffffu, lng);
    if (m) {
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(longCount, __popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (lng) longList[base + __popc(m & ((1u << lane) - 1u))] = i;
    }
}
__global__ void k_segment_sort_long(const int* off, const int* cnt, int* partners, uint64_t* keys, const int* longList,
                                    const int* longCount) {
    const int lane = threadIdx.x & 31;
    const int nl = *longCount, nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int q = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); q < nl; q += nw) {   // uniform per warp
        const int i = longList[q], o = off[i], c = cnt[i];
        const uint64_t hi = (uint64_t)(unsigned)i << 32;
        unsigned* p = (unsigned*)partners + o;
        if (c <= 32) {
            unsigned v = lane < c ? p[lane] : 0xffffffffu;
            for (int k = 2; k <= 32; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    const unsigned u = __shfl_xor_sync(0xffffffffu, v, j);
                    v = (((lane & j) == 0) == ((lane & k) == 0)) ? min(v, u) : max(v, u);
                }
            if (lane < c) keys[o + lane] = hi | v;
        } else {
            if (lane == 0)
                for (int gap = c / 2; gap > 0; gap /= 2)   // Shell sort for rare crowded owners
                    for (int k = gap; k < c; k++) {
                        const unsigned x = p[k];
                        int j = k;
                        while (j >= gap && p[j - gap] > x) { p[j] = p[j - gap]; j -= gap; }
                        p[j] = x;
                    }
            __syncwarp();
            for (int k = lane; k < c; k += 32) keys[o + k] = hi | p[k];
            __syncwarp();
        }
    }
}

// Carry manifolds of persisting pairs (binary search in last step's sorted keys: within the
// owner's segment when last step's per-owner offsets are at hand, else over all of them).
__global__ void k_persist(DevWorld w, DevPairs nw, DevPairs old, int nNew, int nOld, const int* offPrev, const int* newCnt,
                          const int* oldCnt) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (newCnt) nNew = min(nNew, *newCnt);
    if (oldCnt) nOld = min(nOld, *oldCnt);
    if (p >= nNew) return;
    uint64_t key = nw.keys[p];
    int lo = 0, hi = nOld - 1, found = -1;
    if (offPrev) {
        const int o = key_owner(key);
        lo = offPrev[o];
        hi = min(offPrev[o + 1], nOld) - 1;
    }
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        uint64_t k = old.keys[mid];
        if (k == key) { found = mid; break; }
        if (k < key) lo = mid + 1; else hi = mid - 1;
    }
    int a = key_owner(key), b = key_partner(key);
    if (found >= 0 && old.has[found]) {
        int n = old.n[found];
        nw.has[p] = 1;
        nw.n[p] = n;
        nw.b0[p] = old.b0[found];
        nw.b1[p] = old.b1[found];
        for (int j = 0; j < n; j++) {
            int s = found * 4 + j, d = p * 4 + j;
            nw.pA[d] = old.pA[s]; nw.pB[d] = old.pB[s]; nw.wA[d] = old.wA[s]; nw.wB[d] = old.wB[s];
            nw.nrm[d] = old.nrm[s]; nw.imp[d] = old.imp[s]; nw.d1[d] = old.d1[s]; nw.d2[d] = old.d2[s];
        }
    } else {
        nw.has[p] = 0;
        nw.n[p] = 0;
        int mb0, mb1;
        manifold_bodies(a, b, w.sh.type[w.shape[min(a, b)]], w.sh.type[w.shape[max(a, b)]], mb0, mb1);
        nw.b0[p] = mb0;
        nw.b1[p] = mb1;
    }
}

static inline int gridn(int n, int b) { return (n + b - 1) / b; }

// The tree over the Morton order is rebuilt every rebuildInterval steps and only refitted to the
// new AABBs in between: a refitted tree bounds every body exactly, so the traversal finds the
// same pair set whatever the tree's shape; only its cost depends on how stale the order is.
// The tree over the finite bodies' current w.amin/w.amax: Morton keys of the box centres (the
// batch world in the high bits), radix sort, world leaf ranges, Karras topology.  Boxes are
// written by a refit.
void broadphase_build_tree(const DevWorld& w, BroadphaseBuffers& bb, cudaStream_t s) {
    const int n = w.nBodies, nf = bb.nFinite;
    bb.built = true;
    bb.sinceBuild = 0;
    cudaMemsetAsync(bb.bounds, 0, sizeof(unsigned) * 6, s);
    cudaMemsetAsync(bb.bounds, 0xff, sizeof(unsigned) * 3, s);
    k_bounds<<<gridn(n, 256), 256, 0, s>>>(w, bb.bounds); note_launch();
    k_morton<<<gridn(n, 256), 256, 0, s>>>(w, bb.bounds, bb.mkeys, bb.sortedBody); note_launch();
    radix_sort_pairs(bb.mkeys, bb.sortedBody, bb.mkeys_alt, bb.vals_alt, n, 32 + bb.worldBits, bb.sortScratch, s);
    if (nf > 0) {
        cudaMemsetAsync(bb.wstart, 0xff, sizeof(int) * bb.nWorlds, s);
        cudaMemsetAsync(bb.wend, 0xff, sizeof(int) * bb.nWorlds, s);
        cudaMemsetAsync(bb.wroot, 0xff, sizeof(int) * bb.nWorlds, s);
        k_world_ranges<<<gridn(nf, 256), 256, 0, s>>>(bb.mkeys, nf, bb.wstart, bb.wend, bb.wroot); note_launch();
        if (nf > 1) {
            cudaMemsetAsync(bb.bvh.parent, 0xff, sizeof(int) * (nf - 1), s);
            cudaMemsetAsync(bb.bvh.leafParent, 0xff, sizeof(int) * nf, s);   // single-leaf worlds keep -1
            k_karras<<<gridn(nf - 1, 256), 256, 0, s>>>(bb.mkeys, nf, bb.bvh, bb.wstart, bb.wend, bb.wroot); note_launch();
        }
    }
}

// Refit of the current tree topology over the boxes in wq.amin / wq.amax into another node
// record array (the broadphase's own records are left as they are).
void broadphase_refit_into(const DevWorld& wq, const BroadphaseBuffers& bb, float4* node, int* visit, cudaStream_t s) {
    const int nf = bb.nFinite;
    if (nf < 2) return;
    Bvh t = bb.bvh;
    t.node = node;
    t.visit = visit;
    cudaMemsetAsync(visit, 0, sizeof(int) * (nf - 1), s);
    k_refit<<<gridn(nf, 256), 256, 0, s>>>(wq, bb.sortedBody, nf, t); note_launch();
}

void broadphase_run_count(const DevWorld& w, BroadphaseBuffers& bb, cudaStream_t s) {
    int n = w.nBodies;
    if (bb.built && bb.sinceBuild + 1 < bb.rebuildInterval) {
        bb.sinceBuild++;
        int nf = bb.nFinite;
        cudaMemsetAsync(bb.cnt, 0, sizeof(int) * (n + 1), s);
        if (nf > 1) {
            cudaMemsetAsync(bb.bvh.visit, 0, sizeof(int) * (nf - 1), s);
            k_refit<<<gridn(nf, 256), 256, 0, s>>>(w, bb.sortedBody, nf, bb.bvh); note_launch();
            k_traverse<false><<<gridn(nf, 128), 128, 0, s>>>(w, bb.sortedBody, nf, bb.bvh, bb.wroot, bb.cnt, nullptr,
                                                              nullptr, nullptr, 0, bb.tcount, bb.tcache); note_launch();
        }
        cudaMemsetAsync(bb.candBound, 0, sizeof(int), s);
        if (bb.nPlanes > 0)
            k_plane_pairs<false><<<gridn(n, 256), 256, 0, s>>>(w, bb.planeList, bb.planeStart, bb.cnt, nullptr, nullptr,
                                                                nullptr, 0, bb.candBound); note_launch();
        exclusive_scan(bb.cnt, bb.off, bb.total, n + 1, bb.scanScratch, s);
        return;
    }
    broadphase_build_tree(w, bb, s);
    int nf = bb.nFinite;
    cudaMemsetAsync(bb.cnt, 0, sizeof(int) * (n + 1), s);
    if (nf > 0) {
        if (nf > 1) {
            cudaMemsetAsync(bb.bvh.visit, 0, sizeof(int) * (nf - 1), s);
            k_refit<<<gridn(nf, 256), 256, 0, s>>>(w, bb.sortedBody, nf, bb.bvh); note_launch();
            k_traverse<false><<<gridn(nf, 128), 128, 0, s>>>(w, bb.sortedBody, nf, bb.bvh, bb.wroot, bb.cnt, nullptr,
                                                              nullptr, nullptr, 0, bb.tcount, bb.tcache); note_launch();
        }
    }
    cudaMemsetAsync(bb.candBound, 0, sizeof(int), s);
    if (bb.nPlanes > 0)
        k_plane_pairs<false><<<gridn(n, 256), 256, 0, s>>>(w, bb.planeList, bb.planeStart, bb.cnt, nullptr, nullptr,
                                                            nullptr, 0, bb.candBound); note_launch();
    exclusive_scan(bb.cnt, bb.off, bb.total, n + 1, bb.scanScratch, s);
}

void broadphase_run_fill(const DevWorld& w, BroadphaseBuffers& bb, DevPairs& nw, int capacity, cudaStream_t s) {
    int n = w.nBodies, nf = bb.nFinite;
    cudaMemsetAsync(bb.cursor, 0, sizeof(int) * (n + 1), s);
    // counts are recovered from the offsets: cnt[i] = off[i+1] - off[i]
    if (nf > 1)
        k_traverse<true><<<gridn(nf, 128), 128, 0, s>>>(w, bb.sortedBody, nf, bb.bvh, bb.wroot, nullptr, bb.off,
                                                         bb.cursor, bb.partners, capacity, bb.tcount, bb.tcache); note_launch();
    if (bb.nPlanes > 0)
        k_plane_pairs<true><<<gridn(n, 256), 256, 0, s>>>(w, bb.planeList, bb.planeStart, nullptr, bb.off, bb.cursor,
                                                           bb.partners, capacity, nullptr); note_launch();
    if (w.hasCompound) {
        k_segment_sort<<<gridn(n, 128), 128, 0, s>>>(w, n, bb.off, bb.cursor, bb.partners, nw.keys, capacity);
    } else {
        // the long segments' owners are listed in tcount, which the filling traversal has read
        cudaMemsetAsync(bb.segLong, 0, sizeof(int), s);
        k_segment_sort_short<<<gridn(n, 128), 128, 0, s>>>(n, bb.off, bb.cursor, bb.partners, nw.keys, capacity,
                                                            bb.tcount, bb.segLong);
        note_launch();
        k_segment_sort_long<<<std::min(gridn(n, 4), 1024), 128, 0, s>>>(bb.off, bb.cursor, bb.partners, nw.keys,
                                                                        bb.tcount, bb.segLong);
    }
    note_launch();
}

void broadphase_persist(const DevWorld& w, BroadphaseBuffers& bb, DevPairs& nw, const DevPairs& old, int nNew, int nOld,
                        cudaStream_t s, const int* newCnt, const int* oldCnt) {
    if (nNew > 0) {
        k_persist<<<gridn(nNew, 256), 256, 0, s>>>(w, nw, old, nNew, nOld, bb.offPrevValid ? bb.offPrev : nullptr, newCnt,
                                                    oldCnt);
        note_launch();
    }
    std::swap(bb.off, bb.offPrev);   // this step's offsets index the pair array the next step persists from
    bb.offPrevValid = true;
}

}  // namespace jbg
