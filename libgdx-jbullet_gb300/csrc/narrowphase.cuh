#pragma once
#include "jbgpu_internal.cuh"

namespace jbg {

// EPA queue + scratch arena (per-slot polytopes; see epa.cuh for the slot layout).
struct NarrowBuffers {
    void* queue = nullptr;        // EpaRec per queued pair (pair capacity)
    int* queueCount = nullptr;
    int slots = 0;                // concurrent EPA threads, each owning one slot
    float4 *fN = nullptr, *mW = nullptr, *mR = nullptr, *seen = nullptr;
    int4 *fV = nullptr, *fF = nullptr, *fE = nullptr;
    float* fD = nullptr;
    int2* stack = nullptr;
};

size_t epa_queue_record_bytes();
void narrowphase_launch(const DevWorld& w, DevPairs& P, int nPairs, NarrowBuffers& nb, cudaStream_t s,
                        const Prof* prof = nullptr);

}  // namespace jbg
