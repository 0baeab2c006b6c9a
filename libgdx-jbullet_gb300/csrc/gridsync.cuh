// Grid-wide barrier of the library's cooperative kernels (all blocks co-resident).
#pragma once
#include "jbgpu_internal.cuh"

namespace jbg {

// ---- grid barrier (bounded wait) -----------------------------------------------------------
// Arrival by an acquire-release atomic on a count that grows through the launch, acquire
// polling of the count.  A wait gives up after a bounded number of polls and sets ST_TIMEOUT (the host
// reports JBGPU_ERR_TIMEOUT); once the flag is set every later barrier returns at once.
constexpr long long BARRIER_SPIN_LIMIT = 20000000;

__device__ __forceinline__ unsigned ld_acquire(const int* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned atom_add_acq_rel(int* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void st_release(int* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void red_release_add(int* p, int v) {
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// `passed` counts the arrivals of all blocks up to this barrier (thread 0 keeps it; every block
// passes the same barriers).  The arrival is a fire-and-forget release add, so a block waits for
// one round trip (its polls) rather than its atomic's return and then a poll.
__device__ __forceinline__ void grid_barrier(int* ctr, int nblocks, unsigned& passed) {
    __syncthreads();
    if (threadIdx.x == 0) {
        passed += (unsigned)nblocks;
        red_release_add(&ctr[C_BAR_COUNT], 1);
        long long spins = 0;
        while (ld_acquire(&ctr[C_BAR_COUNT]) < passed) {
            if ((++spins & 31) == 0 && (spins > BARRIER_SPIN_LIMIT || (ld_acquire(&ctr[C_STATUS]) & ST_TIMEOUT))) {
                atomicOr(&ctr[C_STATUS], ST_TIMEOUT);
                break;
            }
        }
    }
    __syncthreads();
}

}  // namespace jbg
