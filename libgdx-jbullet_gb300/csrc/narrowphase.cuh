#pragma once
#include "../../include/jbgpu.h"
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

// Narrowphase whose EPA pass uses scratch compiled into the library (no allocation).
constexpr int STATIC_EPA_SLOTS = JBGPU_STATIC_EPA_SLOTS_MAX;   // EPA threads that can run at once on it
constexpr int MAX_STATIC_DEVICES = 64;
size_t epa_static_scratch_bytes();
// Device address of the static scratch on `device`, which must be current; looked up once per
// device and cached.  Returns 0 on success.
int epa_static_scratch(int device, void** base);
void narrowphase_launch_static(const DevWorld& w, DevPairs& P, int nPairs, NarrowBuffers& nb, void* base, int slots,
                               cudaStream_t s);

}  // namespace jbg
