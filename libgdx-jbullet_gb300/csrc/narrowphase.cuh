#pragma once
#include "../../include/jbgpu.h"
#include "jbgpu_internal.cuh"

namespace jbg {

constexpr int NB_BUCKETS = 11;   // narrowphase algorithm buckets (pairs grouped by them)

// EPA queue (the polytopes live in shared memory, one warp and one polytope per block).
struct NarrowBuffers {
    void* queue = nullptr;        // EpaRec per queued pair (pair capacity)
    int* queueCount = nullptr;
    int slots = 0;                // EPA blocks, striding over the queue
    int* ovfQueue = nullptr;      // queries the 192-face tier left to the full-capacity tier
    int* ovfCount = nullptr;      // 3 ints: that list's count, ovfQueue2's count, the tier mode
    int* ovfQueue2 = nullptr;     // queries the 96-face tier left to the 192-face tier
    unsigned char* pairBucket = nullptr;   // algorithm bucket per pair (pair capacity)
    int* perm = nullptr;          // pairs grouped by bucket (pair capacity)
    int* blockOff = nullptr;      // per block and bucket counts, scanned in place (NB_BUCKETS x pair blocks)
    bool group = true;            // group pairs by algorithm (worth it with two or more shape kinds)
    void* scanScratch = nullptr;  // scan scratch for blockOff
    // concave pass (worlds with triangle meshes): per pair its candidate triangle count and
    // offset, the (pair, triangle) candidates, their GJK/EPA results (2 float4 each) and the
    // candidates' own EPA queue with its overflow lists and counters (queue count, two overflow
    // counts, tier mode)
    int* meshCnt = nullptr;
    int* meshOff = nullptr;
    int* meshList = nullptr;      // [0]: mesh pairs this step, then their pair indices
    int* meshTotal = nullptr;
    void* meshScan = nullptr;
    int capMeshPairs = 0;
    int2* cand = nullptr;
    float4* candRes = nullptr;
    void* candQueue = nullptr;
    int* candOvf = nullptr;
    int* candOvf2 = nullptr;
    int* candCount = nullptr;
    int capCand = 0;
};

size_t epa_queue_record_bytes();
int narrowphase_configure();      // once per world: the EPA kernel's shared-memory size
// cntp (nullable): the pair count on the device; nPairs is then an upper bound (graph replays).
void narrowphase_launch(const DevWorld& w, DevPairs& P, int nPairs, NarrowBuffers& nb, cudaStream_t s,
                        const Prof* prof = nullptr, const int* cntp = nullptr);

// The concave pass (after narrowphase_launch, in a world with triangle meshes).
// concave_launch reads the exact candidate count back to the host (hostTotal: a pinned int) and
// grows its buffers (the stage path); concave_launch_bounded runs on buffers reserved beforehand
// for the bound the step's pair count pass computed (candBound), every count read on the device,
// so that it can be captured in a graph.  Both return nonzero when a CUDA call failed.
// concave_reserve: -1 allocation failed, 1 a buffer moved, 0 nothing changed.
int concave_reserve(NarrowBuffers& nb, int pairCap, int candCap, cudaStream_t s);
int concave_launch(const DevWorld& w, DevPairs& P, int nPairs, const int* cntp, NarrowBuffers& nb, int* hostTotal,
                   cudaStream_t s);
int concave_launch_bounded(const DevWorld& w, DevPairs& P, int nPairs, const int* cntp, NarrowBuffers& nb, int candBound,
                           cudaStream_t s);
void concave_free(NarrowBuffers& nb);

// Narrowphase whose EPA pass uses scratch compiled into the library (no allocation).
constexpr int STATIC_EPA_SLOTS = JBGPU_STATIC_EPA_SLOTS_MAX;   // EPA warps that can run at once on it
constexpr int MAX_STATIC_DEVICES = 64;
size_t epa_static_scratch_bytes();
// Device address of the static scratch on `device`, which must be current; looked up once per
// device and cached.  Returns 0 on success.
int epa_static_scratch(int device, void** base);
void narrowphase_launch_static(const DevWorld& w, DevPairs& P, int nPairs, NarrowBuffers& nb, void* base, int slots,
                               cudaStream_t s);

}  // namespace jbg
