// Per-contact MLP of the learned warm start: 24 -> 64 -> 64 -> 3, GELU (tanh form), BF16
// weights and activations into the tensor cores (mma.sync m16n8k16, FP32 accumulate), FP32
// elementwise work.  A block handles 64 samples with 4 warps; every matrix product of the
// forward and backward passes is one call of warp_gemm over operands staged in shared memory.
#pragma once
#include <cuda_bf16.h>
#include "../../include/jbgpu.h"
#include "jbgpu_internal.cuh"

namespace jbg {

constexpr int MLP_IN = 24, MLP_INP = 32;     // inputs, padded to two k-steps
constexpr int MLP_H = 64;
constexpr int MLP_OUT = 3, MLP_OUTP = 16;   // outputs, padded for the transposed products
constexpr int MLP_TILE = 64;                // samples per block
constexpr int MLP_THREADS = 128;
// parameter packing (FP32 master copy): W1[64][24] b1[64] W2[64][64] b2[64] W3[3][64] b3[3]
constexpr int MLP_OFF_W1 = 0, MLP_OFF_B1 = MLP_OFF_W1 + MLP_H * MLP_IN, MLP_OFF_W2 = MLP_OFF_B1 + MLP_H,
              MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H, MLP_OFF_W3 = MLP_OFF_B2 + MLP_H,
              MLP_OFF_B3 = MLP_OFF_W3 + MLP_OUT * MLP_H, MLP_NPARAM = MLP_OFF_B3 + MLP_OUT;
// normalisation block: x' = asinh((x - inMean) * inScale);  y = y' * outScale + outMean; then
// the impulse unit (impulse that stops one step of gravity for unit inverse mass) used by the
// warm-start transform
constexpr int MLP_NORM = 2 * MLP_IN + 2 * MLP_OUT + 1;
constexpr int MLP_NORM_UNIT = 2 * MLP_IN + 2 * MLP_OUT;

JBD float mlp_norm_in(const float* norm, int k, float x) { return asinhf((x - norm[k]) * norm[MLP_IN + k]); }

// The warm-start outputs are relative impulse corrections r, carried by the network as
// asinh(r / MLP_REL) so that the many small corrections and the few large ones both matter.
constexpr float MLP_REL = 0.01f;

struct MlpDev {
    const __nv_bfloat16* w1;   // [64][32] (k >= 24 zero)
    const __nv_bfloat16* w2;   // [64][64]
    const __nv_bfloat16* w3;   // [16][64] (rows >= 3 zero)
    const float* p;            // FP32 parameters (biases read from here)
    const float* norm;         // MLP_NORM floats
};

MlpDev mlp_view(const jbgpu_mlp* h);   // mlp.cu

// Shared-memory working set of one 64-sample block.
struct MlpSmem {
    __nv_bfloat16 x[MLP_TILE][MLP_INP];
    float z1[MLP_TILE][MLP_H];
    __nv_bfloat16 h1[MLP_TILE][MLP_H];
    float z2[MLP_TILE][MLP_H];
    __nv_bfloat16 h2[MLP_TILE][MLP_H];
    float y[MLP_TILE][4];
    __nv_bfloat16 dy[MLP_TILE][MLP_OUTP];
    __nv_bfloat16 dz2[MLP_TILE][MLP_H];
    __nv_bfloat16 dz1[MLP_TILE][MLP_H];
    __nv_bfloat16 w1[MLP_H][MLP_INP];
    __nv_bfloat16 w2[MLP_H][MLP_H];
    __nv_bfloat16 w3[MLP_OUTP][MLP_H];
};

JBD uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

JBD void mma_bf16_16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// One warp: C[m0..m0+16) x [n0..n0+8) = sum over k < K of A(i,k) * B(k,n), K a multiple of 16.
// Fragment layout of m16n8k16 (g = lane / 4, t = lane % 4): A regs hold (g, 2t..2t+1),
// (g+8, 2t..), (g, 2t+8..), (g+8, 2t+8..); B regs (k = 2t..2t+1, n = g), (k = 2t+8.., n = g);
// C holds (g, 2t), (g, 2t+1), (g+8, 2t), (g+8, 2t+1).
template <class FA, class FB>
JBD void warp_gemm(float c[4], int m0, int n0, int K, FA A, FB B) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    c[0] = c[1] = c[2] = c[3] = 0.0f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[4], b[2];
        a[0] = pack_bf16(A(m0 + g, k0 + 2 * t), A(m0 + g, k0 + 2 * t + 1));
        a[1] = pack_bf16(A(m0 + g + 8, k0 + 2 * t), A(m0 + g + 8, k0 + 2 * t + 1));
        a[2] = pack_bf16(A(m0 + g, k0 + 2 * t + 8), A(m0 + g, k0 + 2 * t + 9));
        a[3] = pack_bf16(A(m0 + g + 8, k0 + 2 * t + 8), A(m0 + g + 8, k0 + 2 * t + 9));
        b[0] = pack_bf16(B(k0 + 2 * t, n0 + g), B(k0 + 2 * t + 1, n0 + g));
        b[1] = pack_bf16(B(k0 + 2 * t + 8, n0 + g), B(k0 + 2 * t + 9, n0 + g));
        mma_bf16_16816(c, a, b);
    }
}

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))), and its derivative.
JBD float gelu(float x) {
    const float k = 0.7978845608028654f;
    float u = k * (x + 0.044715f * x * x * x);
    return 0.5f * x * (1.0f + tanhf(u));
}
JBD float gelu_grad(float x) {
    const float k = 0.7978845608028654f;
    float u = k * (x + 0.044715f * x * x * x);
    float th = tanhf(u);
    return 0.5f * (1.0f + th) + 0.5f * x * (1.0f - th * th) * k * (1.0f + 3.0f * 0.044715f * x * x);
}

// Weights into shared memory (all threads of the block).
JBD void mlp_load_weights(MlpSmem& S, const MlpDev& M) {
    for (int i = threadIdx.x; i < MLP_H * MLP_INP; i += blockDim.x) S.w1[i / MLP_INP][i % MLP_INP] = M.w1[i];
    for (int i = threadIdx.x; i < MLP_H * MLP_H; i += blockDim.x) S.w2[i / MLP_H][i % MLP_H] = M.w2[i];
    for (int i = threadIdx.x; i < MLP_OUTP * MLP_H; i += blockDim.x) S.w3[i / MLP_H][i % MLP_H] = M.w3[i];
}

// Forward pass over S.x (normalised inputs, bf16): S.z1/h1, S.z2/h2, S.y (normalised outputs).
// Warp w owns samples [16w, 16w+16).  Ends with a block barrier.
JBD void mlp_forward(MlpSmem& S, const MlpDev& M) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int m0 = warp * 16;
    for (int n0 = 0; n0 < MLP_H; n0 += 8) {
        float c[4];
        warp_gemm(c, m0, n0, MLP_INP, [&](int i, int k) { return S.x[i][k]; }, [&](int k, int n) { return S.w1[n][k]; });
        for (int q = 0; q < 4; q++) {
            int i = m0 + g + (q >> 1) * 8, n = n0 + 2 * t + (q & 1);
            float z = c[q] + M.p[MLP_OFF_B1 + n];
            S.z1[i][n] = z;
            S.h1[i][n] = __float2bfloat16_rn(gelu(z));
        }
    }
    __syncwarp();
    for (int n0 = 0; n0 < MLP_H; n0 += 8) {
        float c[4];
        warp_gemm(c, m0, n0, MLP_H, [&](int i, int k) { return S.h1[i][k]; }, [&](int k, int n) { return S.w2[n][k]; });
        for (int q = 0; q < 4; q++) {
            int i = m0 + g + (q >> 1) * 8, n = n0 + 2 * t + (q & 1);
            float z = c[q] + M.p[MLP_OFF_B2 + n];
            S.z2[i][n] = z;
            S.h2[i][n] = __float2bfloat16_rn(gelu(z));
        }
    }
    __syncwarp();
    {
        float c[4];
        warp_gemm(c, m0, 0, MLP_H, [&](int i, int k) { return S.h2[i][k]; }, [&](int k, int n) { return S.w3[n][k]; });
        for (int q = 0; q < 4; q++) {
            int i = m0 + g + (q >> 1) * 8, n = 2 * t + (q & 1);
            if (n < MLP_OUT) S.y[i][n] = c[q] + M.p[MLP_OFF_B3 + n];
        }
    }
    __syncthreads();
}

}  // namespace jbg
