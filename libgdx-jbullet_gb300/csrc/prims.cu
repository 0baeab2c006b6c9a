// Exclusive scan and stable LSD radix sort (8-bit digits) for the broadphase.
//
// Radix pass = three kernels: per-tile digit histograms (shared-memory atomics), one
// single-block exclusive scan over the digit-major histogram table, and a scatter that
// ranks keys stably inside each tile with warp match masks and writes them to their
// global digit offsets.  Tiles are 4096 keys (256 threads x 16 rounds).
#include <cuda_runtime.h>
#include "prims.cuh"

namespace jbg {

namespace {
constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;
constexpr int RS_BINS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
}

// Block-wide inclusive scan of one int per thread (blockDim = 1024).
__device__ __forceinline__ int block_inclusive_scan(int v, int* smem) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) smem[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int x = (lane < (int)(blockDim.x >> 5)) ? smem[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        smem[lane] = x;
    }
    __syncthreads();
    if (wid > 0) v += smem[wid - 1];
    __syncthreads();
    return v;
}

__global__ void k_scan_tiles(const int* in, int* out, int* tileSums, int n) {
    __shared__ int smem[32];
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int sum = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) { v[k] = (base + k < n) ? in[base + k] : 0; sum += v[k]; }
    int incl = block_inclusive_scan(sum, smem);
    int run = incl - sum;
    for (int k = 0; k < SCAN_ITEMS; k++) { if (base + k < n) out[base + k] = run; run += v[k]; }
    if (threadIdx.x == blockDim.x - 1) tileSums[blockIdx.x] = incl;
}

// Single block: exclusive scan of m values in place (m arbitrary, looped in chunks of 1024).
__global__ void k_scan_single(int* data, int m, int* total) {
    __shared__ int smem[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < m; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = (i < m) ? data[i] : 0;
        int incl = block_inclusive_scan(v, smem);
        int c = carry;
        if (i < m) data[i] = c + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = c + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_add(int* out, const int* tileSums, int n) {
    int add = tileSums[blockIdx.x];
    int base = blockIdx.x * SCAN_TILE;
    for (int k = threadIdx.x; k < SCAN_TILE; k += blockDim.x)
        if (base + k < n) out[base + k] += add;
}

size_t scan_scratch_bytes(int n) { return sizeof(int) * (size_t)((n + SCAN_TILE - 1) / SCAN_TILE + 1); }

void exclusive_scan(const int* in, int* out, int* total, int n, void* scratch, cudaStream_t s) {
    if (n <= 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(int), s);
        return;
    }
    int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    int* sums = (int*)scratch;
    k_scan_tiles<<<tiles, SCAN_BLOCK, 0, s>>>(in, out, sums, n); note_launch();
    k_scan_single<<<1, SCAN_BLOCK, 0, s>>>(sums, tiles, total); note_launch();
    if (tiles > 1) { k_scan_add<<<tiles, 256, 0, s>>>(out, sums, n); note_launch(); }
}

// ---- radix sort ---------------------------------------------------------------------------
__global__ void k_rs_hist(const uint64_t* keys, int n, int shift, int* hist, int tiles) {
    __shared__ int bins[RS_BINS];
    bins[threadIdx.x] = 0;
    __syncthreads();
    int base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; r++) {
        int i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&bins[(int)((keys[i] >> shift) & 0xff)], 1);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = bins[threadIdx.x];   // digit-major
}

__global__ void k_rs_scatter(const uint64_t* keys, const int* vals, uint64_t* okeys, int* ovals, int n, int shift,
                             const int* hist, int tiles) {
    __shared__ int warpCnt[RS_WARPS][RS_BINS];
    __shared__ int digitBase[RS_BINS];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    digitBase[threadIdx.x] = hist[threadIdx.x * tiles + blockIdx.x];
    const unsigned lt = (1u << lane) - 1u;
    int base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; r++) {
        for (int k = threadIdx.x; k < RS_WARPS * RS_BINS; k += RS_THREADS) (&warpCnt[0][0])[k] = 0;
        __syncthreads();
        int i = base + r * RS_THREADS + threadIdx.x;
        bool valid = i < n;
        uint64_t key = valid ? keys[i] : 0;
        int d = valid ? (int)((key >> shift) & 0xff) : RS_BINS;   // invalid lanes form their own group
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rankInWarp = __popc(peers & lt);
        if (valid && rankInWarp == 0) warpCnt[wid][d] = __popc(peers);
        __syncthreads();
        {   // per digit: exclusive prefix over warps, advance the digit base
            int dgt = threadIdx.x;
            int run = digitBase[dgt];
            for (int wv = 0; wv < RS_WARPS; wv++) { int c = warpCnt[wv][dgt]; warpCnt[wv][dgt] = run; run += c; }
            digitBase[dgt] = run;
        }
        __syncthreads();
        if (valid) {
            int pos = warpCnt[wid][d] + rankInWarp;
            okeys[pos] = key;
            ovals[pos] = vals[i];
        }
        __syncthreads();
    }
}

size_t sort_scratch_bytes(int n) {
    int tiles = (n + RS_TILE - 1) / RS_TILE;
    return sizeof(int) * ((size_t)tiles * RS_BINS + 16) + scan_scratch_bytes(tiles * RS_BINS);
}

void radix_sort_pairs(uint64_t* keys, int* vals, uint64_t* keys_alt, int* vals_alt, int n, int bits, void* scratch,
                      cudaStream_t s) {
    if (n <= 1) return;
    int tiles = (n + RS_TILE - 1) / RS_TILE;
    int* hist = (int*)scratch;
    void* scanScratch = (void*)(hist + (size_t)tiles * RS_BINS + 16);
    int passes = (bits + 7) / 8;
    uint64_t *ka = keys, *kb = keys_alt;
    int *va = vals, *vb = vals_alt;
    for (int p = 0; p < passes; p++) {
        int shift = 8 * p;
        k_rs_hist<<<tiles, RS_THREADS, 0, s>>>(ka, n, shift, hist, tiles); note_launch();
        exclusive_scan(hist, hist, nullptr, tiles * RS_BINS, scanScratch, s);
        k_rs_scatter<<<tiles, RS_THREADS, 0, s>>>(ka, va, kb, vb, n, shift, hist, tiles); note_launch();
        uint64_t* tk = ka; ka = kb; kb = tk;
        int* tv = va; va = vb; vb = tv;
    }
    if (ka != keys) {
        cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, s);
    }
}

}  // namespace jbg
