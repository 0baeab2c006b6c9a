#pragma once
#include "jbgpu_internal.cuh"

namespace jbg {

constexpr int LEAF_FLAG = 0x40000000;

struct Bvh {           // Karras radix tree over nf sorted leaves; internal nodes 0..nf-2
    int* left;
    int* right;        // child index, LEAF_FLAG set for leaves
    int* lo;
    int* hi;           // sorted-leaf range covered by the node
    int* parent;       // internal node parents (-1 at roots)
    int* leafParent;
    int* visit;        // refit arrival counters
    // per internal node, 4 float4: left child's box min with the child index in .w, its box max
    // with the child's last sorted leaf in .w, then the same for the right child (one 64-byte
    // record read per visited node)
    float4* node;
};

constexpr int TRAV_CACHE = 64;         // pairs a counting traversal keeps for the filling one

struct BroadphaseBuffers {
    int nFinite = 0, nPlanes = 0, nWorlds = 1, worldBits = 0;
    int rebuildInterval = 1;             // rebuild the tree every this many steps, refit in between
    int sinceBuild = 0;                  // steps since the last build
    bool built = false;                  // the tree matches the current body set
    unsigned* bounds = nullptr;          // 6 ordered-int scene bounds
    uint64_t* mkeys = nullptr;           // morton keys (sorted in place)
    uint64_t* mkeys_alt = nullptr;
    int* sortedBody = nullptr;           // body of each sorted leaf
    int* vals_alt = nullptr;
    void* sortScratch = nullptr;
    void* scanScratch = nullptr;
    Bvh bvh{};
    int* wstart = nullptr;               // per world sorted-leaf range and root
    int* wend = nullptr;
    int* wroot = nullptr;
    int* planeList = nullptr;            // plane bodies grouped by world
    int* planeStart = nullptr;           // nWorlds + 1 offsets into planeList
    int* cnt = nullptr;                  // pairs per owner (n + 1)
    int* off = nullptr;                  // exclusive scan of cnt (n + 1); off[n] = total
    int* offPrev = nullptr;              // last step's off: the old pairs of owner o are [offPrev[o], offPrev[o + 1])
    bool offPrevValid = false;           // offPrev matches the previous pair array
    int* cursor = nullptr;               // fill cursors (n + 1)
    int* total = nullptr;                // device total pair count
    int* segLong = nullptr;              // device: owners whose partner segments the warp pass sorts
    int* candBound = nullptr;            // device: the concave pass's candidates, bounded by the count pass
    int* partners = nullptr;             // CSR partner lists (pair capacity)
    int* tcount = nullptr;               // per sorted leaf: pairs its counting traversal found
    int* tcache = nullptr;               // per sorted leaf: the first TRAV_CACHE partners' sorted leaves
};

void broadphase_build_tree(const DevWorld& w, BroadphaseBuffers& bb, cudaStream_t s);
void broadphase_refit_into(const DevWorld& wq, const BroadphaseBuffers& bb, float4* node, int* visit, cudaStream_t s);
void broadphase_run_count(const DevWorld& w, BroadphaseBuffers& bb, cudaStream_t s);
void broadphase_run_fill(const DevWorld& w, BroadphaseBuffers& bb, DevPairs& nw, int capacity, cudaStream_t s);
// newCnt / oldCnt (nullable): the pair counts on the device, nNew / nOld then being upper bounds.
void broadphase_persist(const DevWorld& w, BroadphaseBuffers& bb, DevPairs& nw, const DevPairs& old, int nNew, int nOld,
                        cudaStream_t s, const int* newCnt = nullptr, const int* oldCnt = nullptr);

}  // namespace jbg
