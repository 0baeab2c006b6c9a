// Device-wide primitives written for this library: exclusive scan of int32 and a stable
// least-significant-digit radix sort of (uint64 key, int32 value) pairs.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace jbg {

// Counts a kernel launch of this library (process-wide, reported by jbgpu_launch_count).
void note_launch();

// Scratch sizes (bytes) for n elements.
size_t scan_scratch_bytes(int n);
size_t sort_scratch_bytes(int n);

// out[i] = sum(in[0..i-1]); total (device, may be null) = sum(in[0..n-1]).  in == out allowed.
void exclusive_scan(const int* in, int* out, int* total, int n, void* scratch, cudaStream_t s);

// Sorts keys/vals by the low `bits` bits of the key (stable).  Results end in keys/vals;
// keys_alt/vals_alt are same-sized ping-pong buffers.
void radix_sort_pairs(uint64_t* keys, int* vals, uint64_t* keys_alt, int* vals_alt, int n, int bits, void* scratch,
                      cudaStream_t s);

}  // namespace jbg
