// Training and evaluation of the warm-start MLP (the C ABI jbgpu_mlp_* of include/jbgpu.h):
// mini-batch Adam on mean squared error of normalised targets, with the forward and backward
// products on the tensor cores (mlp.cuh) and FP32 gradients accumulated with atomics.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/jbgpu.h"
#include "mlp.cuh"

namespace jbg {
int set_last_error(int code, const char* msg);   // world.cu
}
using namespace jbg;

struct jbgpu_mlp {
    int device = 0;
    cudaStream_t s = nullptr;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr, *norm = nullptr, *loss = nullptr;
    __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w3 = nullptr;
    float *X = nullptr, *T = nullptr;     // training set on the device
    int n = 0, cap = 0;
    int* idx = nullptr;                   // epoch permutation
    long long adamStep = 0;
    float* io = nullptr;                  // staging for forward / gradients (capacity ioCap samples)
    int ioCap = 0;
};

namespace jbg {

MlpDev mlp_view(const jbgpu_mlp* h) {
    MlpDev d;
    d.w1 = h->w1;
    d.w2 = h->w2;
    d.w3 = h->w3;
    d.p = h->p;
    d.norm = h->norm;
    return d;
}

// FP32 parameters -> padded BF16 weight copies.
__global__ void k_mlp_pack(const float* p, __nv_bfloat16* w1, __nv_bfloat16* w2, __nv_bfloat16* w3) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < MLP_H * MLP_INP) {
        int r = i / MLP_INP, c = i % MLP_INP;
        w1[i] = __float2bfloat16_rn(c < MLP_IN ? p[MLP_OFF_W1 + r * MLP_IN + c] : 0.0f);
    }
    if (i < MLP_H * MLP_H) w2[i] = __float2bfloat16_rn(p[MLP_OFF_W2 + i]);
    if (i < MLP_OUTP * MLP_H) {
        int r = i / MLP_H, c = i % MLP_H;
        w3[i] = __float2bfloat16_rn(r < MLP_OUT ? p[MLP_OFF_W3 + r * MLP_H + c] : 0.0f);
    }
}

// Normalised sample rows [first, first + 64) of X (through idx when given) into S.x.
JBD int mlp_load_inputs(MlpSmem& S, const MlpDev& M, const float* X, const int* idx, int first, int count) {
    int valid = min(MLP_TILE, count - first);
    for (int e = threadIdx.x; e < MLP_TILE * MLP_INP; e += blockDim.x) {
        int i = e / MLP_INP, k = e % MLP_INP;
        float v = 0.0f;
        if (i < valid && k < MLP_IN) {
            int row = idx ? idx[first + i] : first + i;
            v = mlp_norm_in(M.norm, k, X[(size_t)row * MLP_IN + k]);
        }
        S.x[i][k] = __float2bfloat16_rn(v);
    }
    return valid;
}

// One 64-sample tile of a mini-batch: forward, loss, backward, gradients added into grad.
// coef = 2 / (batch samples x outputs): the derivative of the batch-mean squared error.
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_train(MlpDev M, const float* X, const float* T, const int* idx,
                                                            int first, int count, float coef, float* grad, float* loss) {
    extern __shared__ __align__(16) unsigned char mlpSmem[];
    MlpSmem& S = *reinterpret_cast<MlpSmem*>(mlpSmem);
    const int tileFirst = first + blockIdx.x * MLP_TILE;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int m0 = warp * 16;
    mlp_load_weights(S, M);
    const int valid = mlp_load_inputs(S, M, X, idx, tileFirst, first + count);
    __syncthreads();
    mlp_forward(S, M);
    // loss and dY (FP32 kept in S.y, BF16 copy padded to 16 columns in S.dy)
    float part = 0.0f;
    for (int e = threadIdx.x; e < MLP_TILE * MLP_OUTP; e += blockDim.x) {
        int i = e / MLP_OUTP, o = e % MLP_OUTP;
        float d = 0.0f;
        if (i < valid && o < MLP_OUT) {
            int row = idx ? idx[tileFirst + i] : tileFirst + i;
            float tn = (T[(size_t)row * MLP_OUT + o] - M.norm[2 * MLP_IN + o]) / M.norm[2 * MLP_IN + MLP_OUT + o];
            float r = S.y[i][o] - tn;
            part += r * r;
            d = coef * r;
        }
        S.dy[i][o] = __float2bfloat16_rn(d);
        if (o < MLP_OUT) S.y[i][o] = d;
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0 && part != 0.0f) atomicAdd(loss, part * coef * 0.5f);
    __syncthreads();
    // dW3 = dY^T H2 (16 padded rows x 64), warps split the columns
    for (int n0 = warp * 16; n0 < warp * 16 + 16; n0 += 8) {
        float c[4];
        warp_gemm(c, 0, n0, MLP_TILE, [&](int o, int k) { return S.dy[k][o]; }, [&](int k, int n) { return S.h2[k][n]; });
        for (int q = 0; q < 4; q++) {
            int o = g + (q >> 1) * 8, n = n0 + 2 * t + (q & 1);
            if (o < MLP_OUT) atomicAdd(&grad[MLP_OFF_W3 + o * MLP_H + n], c[q]);
        }
    }
    if (threadIdx.x < MLP_OUT) {
        float sdb = 0.0f;
        for (int i = 0; i < MLP_TILE; i++) sdb += S.y[i][threadIdx.x];
        atomicAdd(&grad[MLP_OFF_B3 + threadIdx.x], sdb);
    }
    // dZ2 = (dY W3) * gelu'(Z2)
    for (int n0 = 0; n0 < MLP_H; n0 += 8) {
        float c[4];
        warp_gemm(c, m0, n0, MLP_OUTP, [&](int i, int k) { return S.dy[i][k]; }, [&](int k, int n) { return S.w3[k][n]; });
        for (int q = 0; q < 4; q++) {
            int i = m0 + g + (q >> 1) * 8, n = n0 + 2 * t + (q & 1);
            S.dz2[i][n] = __float2bfloat16_rn(c[q] * gelu_grad(S.z2[i][n]));
        }
    }
    __syncthreads();
    // dW2 = dZ2^T H1 (rows split over warps), db2
    for (int n0 = 0; n0 < MLP_H; n0 += 8) {
        float c[4];
        warp_gemm(c, m0, n0, MLP_TILE, [&](int i, int k) { return S.dz2[k][i]; }, [&](int k, int n) { return S.h1[k][n]; });
        for (int q = 0; q < 4; q++) {
            int i = m0 + g + (q >> 1) * 8, n = n0 + 2 * t + (q & 1);
            atomicAdd(&grad[MLP_OFF_W2 + i * MLP_H + n], c[q]);
        }
    }
    if (threadIdx.x < MLP_H) {
        float sdb = 0.0f;
        for (int i = 0; i < MLP_TILE; i++) sdb += __bfloat162float(S.dz2[i][threadIdx.x]);
        atomicAdd(&grad[MLP_OFF_B2 + threadIdx.x], sdb);
    }
    // dZ1 = (dZ2 W2) * gelu'(Z1)
    for (int n0 = 0; n0 < MLP_H; n0 += 8) {
        float c[4];
        warp_gemm(c, m0, n0, MLP_H, [&](int i, int k) { return S.dz2[i][k]; }, [&](int k, int n) { return S.w2[k][n]; });
        for (int q = 0; q < 4; q++) {
            int i = m0 + g + (q >> 1) * 8, n = n0 + 2 * t + (q & 1);
            S.dz1[i][n] = __float2bfloat16_rn(c[q] * gelu_grad(S.z1[i][n]));
        }
    }
    __syncthreads();
    // dW1 = dZ1^T X (24 of 32 padded columns), db1
    for (int n0 = 0; n0 < MLP_IN; n0 += 8) {
        float c[4];
        warp_gemm(c, m0, n0, MLP_TILE, [&](int i, int k) { return S.dz1[k][i]; }, [&](int k, int n) { return S.x[k][n]; });
        for (int q = 0; q < 4; q++) {
            int i = m0 + g + (q >> 1) * 8, n = n0 + 2 * t + (q & 1);
            atomicAdd(&grad[MLP_OFF_W1 + i * MLP_IN + n], c[q]);
        }
    }
    if (threadIdx.x < MLP_H) {
        float sdb = 0.0f;
        for (int i = 0; i < MLP_TILE; i++) sdb += __bfloat162float(S.dz1[i][threadIdx.x]);
        atomicAdd(&grad[MLP_OFF_B1 + threadIdx.x], sdb);
    }
}

// Raw features -> raw outputs (y = y' * outScale + outMean) for `count` rows.
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_forward(MlpDev M, const float* X, int count, float* Y) {
    extern __shared__ __align__(16) unsigned char mlpSmem[];
    MlpSmem& S = *reinterpret_cast<MlpSmem*>(mlpSmem);
    mlp_load_weights(S, M);
    for (int first = blockIdx.x * MLP_TILE; first < count; first += gridDim.x * MLP_TILE) {
        const int valid = mlp_load_inputs(S, M, X, nullptr, first, count);
        __syncthreads();
        mlp_forward(S, M);
        for (int e = threadIdx.x; e < valid * MLP_OUT; e += blockDim.x) {
            int i = e / MLP_OUT, o = e % MLP_OUT;
            Y[(size_t)(first + i) * MLP_OUT + o] = S.y[i][o] * M.norm[2 * MLP_IN + MLP_OUT + o] + M.norm[2 * MLP_IN + o];
        }
        __syncthreads();
    }
}

// Adam (bias-corrected step sizes a1 = lr / (1 - b1^t), a2 = 1 / (1 - b2^t)); clears the gradient.
__global__ void k_mlp_adam(float* p, float* g, float* m, float* v, float lr1, float bc2, float b1, float b2, float eps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_NPARAM) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.0f - b1) * gi;
    float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr1 * mi / (sqrtf(vi * bc2) + eps);
    g[i] = 0.0f;
}

size_t mlp_smem_bytes() { return sizeof(MlpSmem); }

}  // namespace jbg

namespace {

#define MCK(x)                                                                 \
    do {                                                                       \
        cudaError_t e_ = (x);                                                  \
        if (e_ != cudaSuccess) return set_last_error(JBGPU_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

int mlp_repack(jbgpu_mlp* h) {
    k_mlp_pack<<<(MLP_H * MLP_H + 255) / 256, 256, 0, h->s>>>(h->p, h->w1, h->w2, h->w3);
    note_launch();
    MCK(cudaGetLastError());
    return JBGPU_OK;
}

int ensure_io(jbgpu_mlp* h, int n) {
    if (n <= h->ioCap) return JBGPU_OK;
    if (h->io) cudaFree(h->io);
    h->io = nullptr;
    MCK(cudaMalloc(&h->io, sizeof(float) * (size_t)n * (MLP_IN + MLP_OUT)));
    h->ioCap = n;
    return JBGPU_OK;
}

void launch_train_batch(jbgpu_mlp* h, const float* X, const float* T, const int* idx, int first, int count) {
    int tiles = (count + MLP_TILE - 1) / MLP_TILE;
    float coef = 2.0f / (float)(count * MLP_OUT);
    k_mlp_train<<<tiles, MLP_THREADS, mlp_smem_bytes(), h->s>>>(mlp_view(h), X, T, idx, first, count, coef, h->g, h->loss);
    note_launch();
}

}  // namespace

extern "C" {

int jbgpu_mlp_create(int32_t device, uint64_t seed, jbgpu_mlp** out) {
    if (!out) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "null out");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return set_last_error(JBGPU_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= ndev) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "bad device ordinal");
    MCK(cudaSetDevice(device));
    jbgpu_mlp* h = new jbgpu_mlp();
    h->device = device;
    auto fail = [&](cudaError_t e) {
        jbgpu_mlp_destroy(h);
        return set_last_error(JBGPU_ERR_CUDA, cudaGetErrorString(e));
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->p, sizeof(float) * MLP_NPARAM)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->g, sizeof(float) * MLP_NPARAM)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->m, sizeof(float) * MLP_NPARAM)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->v, sizeof(float) * MLP_NPARAM)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->norm, sizeof(float) * MLP_NORM)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->loss, sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->w1, sizeof(__nv_bfloat16) * MLP_H * MLP_INP)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->w2, sizeof(__nv_bfloat16) * MLP_H * MLP_H)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&h->w3, sizeof(__nv_bfloat16) * MLP_OUTP * MLP_H)) != cudaSuccess) return fail(e);
    if ((e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem_bytes())) != cudaSuccess)
        return fail(e);
    if ((e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem_bytes())) != cudaSuccess)
        return fail(e);
    // Xavier-uniform weights from a seeded generator, zero biases, identity normalisation
    std::vector<float> p(MLP_NPARAM, 0.0f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fanOut, int fanIn) {
        float a = std::sqrt(6.0f / (float)(fanIn + fanOut));
        std::uniform_real_distribution<float> U(-a, a);
        for (int i = 0; i < fanOut * fanIn; i++) p[off + i] = U(rng);
    };
    fill(MLP_OFF_W1, MLP_H, MLP_IN);
    fill(MLP_OFF_W2, MLP_H, MLP_H);
    fill(MLP_OFF_W3, MLP_OUT, MLP_H);
    std::vector<float> nrm(MLP_NORM, 0.0f);
    for (int k = 0; k < MLP_IN; k++) nrm[MLP_IN + k] = 1.0f;
    for (int o = 0; o < MLP_OUT; o++) nrm[2 * MLP_IN + MLP_OUT + o] = 1.0f;
    nrm[MLP_NORM_UNIT] = 1.0f;
    if ((e = cudaMemcpy(h->p, p.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
    if ((e = cudaMemcpy(h->norm, nrm.data(), sizeof(float) * MLP_NORM, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
    if ((e = cudaMemset(h->g, 0, sizeof(float) * MLP_NPARAM)) != cudaSuccess) return fail(e);
    if ((e = cudaMemset(h->m, 0, sizeof(float) * MLP_NPARAM)) != cudaSuccess) return fail(e);
    if ((e = cudaMemset(h->v, 0, sizeof(float) * MLP_NPARAM)) != cudaSuccess) return fail(e);
    if (mlp_repack(h) != JBGPU_OK || (e = cudaStreamSynchronize(h->s)) != cudaSuccess) return fail(cudaGetLastError());
    *out = h;
    return JBGPU_OK;
}

int jbgpu_mlp_destroy(jbgpu_mlp* h) {
    if (!h) return JBGPU_OK;
    cudaSetDevice(h->device);
    if (h->s) cudaStreamSynchronize(h->s);
    for (void* q : {(void*)h->p, (void*)h->g, (void*)h->m, (void*)h->v, (void*)h->norm, (void*)h->loss, (void*)h->w1,
                    (void*)h->w2, (void*)h->w3, (void*)h->X, (void*)h->T, (void*)h->idx, (void*)h->io})
        if (q) cudaFree(q);
    if (h->s) cudaStreamDestroy(h->s);
    delete h;
    return JBGPU_OK;
}

int jbgpu_mlp_get_params(jbgpu_mlp* h, float* params, float* normalization) {
    if (!h) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "null mlp");
    MCK(cudaSetDevice(h->device));
    MCK(cudaStreamSynchronize(h->s));
    if (params) MCK(cudaMemcpy(params, h->p, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost));
    if (normalization) MCK(cudaMemcpy(normalization, h->norm, sizeof(float) * MLP_NORM, cudaMemcpyDeviceToHost));
    return JBGPU_OK;
}

int jbgpu_mlp_set_params(jbgpu_mlp* h, const float* params, const float* normalization) {
    if (!h) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "null mlp");
    MCK(cudaSetDevice(h->device));
    MCK(cudaStreamSynchronize(h->s));
    if (normalization) {
        for (int o = 0; o < MLP_OUT; o++)
            if (!(normalization[2 * MLP_IN + MLP_OUT + o] != 0.0f))
                return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "output scale must be non-zero");
        MCK(cudaMemcpy(h->norm, normalization, sizeof(float) * MLP_NORM, cudaMemcpyHostToDevice));
    }
    if (params) {
        MCK(cudaMemcpy(h->p, params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice));
        MCK(cudaMemset(h->m, 0, sizeof(float) * MLP_NPARAM));
        MCK(cudaMemset(h->v, 0, sizeof(float) * MLP_NPARAM));
        h->adamStep = 0;
        int rc = mlp_repack(h);
        if (rc) return rc;
    }
    MCK(cudaStreamSynchronize(h->s));
    return JBGPU_OK;
}

int jbgpu_mlp_forward(jbgpu_mlp* h, const float* x, int32_t n, float* y) {
    if (!h || (n > 0 && (!x || !y)) || n < 0) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "bad argument");
    if (n == 0) return JBGPU_OK;
    MCK(cudaSetDevice(h->device));
    int rc = ensure_io(h, n);
    if (rc) return rc;
    float* dx = h->io;
    float* dy = h->io + (size_t)n * MLP_IN;
    MCK(cudaMemcpyAsync(dx, x, sizeof(float) * (size_t)n * MLP_IN, cudaMemcpyHostToDevice, h->s));
    int blocks = std::min((n + MLP_TILE - 1) / MLP_TILE, 1024);
    k_mlp_forward<<<blocks, MLP_THREADS, mlp_smem_bytes(), h->s>>>(mlp_view(h), dx, n, dy);
    note_launch();
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(y, dy, sizeof(float) * (size_t)n * MLP_OUT, cudaMemcpyDeviceToHost, h->s));
    MCK(cudaStreamSynchronize(h->s));
    return JBGPU_OK;
}

int jbgpu_mlp_gradients(jbgpu_mlp* h, const float* x, const float* t, int32_t n, float* grad, float* loss) {
    if (!h || n <= 0 || !x || !t || !grad) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "bad argument");
    MCK(cudaSetDevice(h->device));
    int rc = ensure_io(h, n);
    if (rc) return rc;
    float* dx = h->io;
    float* dt = h->io + (size_t)n * MLP_IN;
    MCK(cudaMemcpyAsync(dx, x, sizeof(float) * (size_t)n * MLP_IN, cudaMemcpyHostToDevice, h->s));
    MCK(cudaMemcpyAsync(dt, t, sizeof(float) * (size_t)n * MLP_OUT, cudaMemcpyHostToDevice, h->s));
    MCK(cudaMemsetAsync(h->g, 0, sizeof(float) * MLP_NPARAM, h->s));
    MCK(cudaMemsetAsync(h->loss, 0, sizeof(float), h->s));
    launch_train_batch(h, dx, dt, nullptr, 0, n);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(grad, h->g, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, h->s));
    float l = 0.0f;
    MCK(cudaMemcpyAsync(&l, h->loss, sizeof(float), cudaMemcpyDeviceToHost, h->s));
    MCK(cudaMemsetAsync(h->g, 0, sizeof(float) * MLP_NPARAM, h->s));
    MCK(cudaStreamSynchronize(h->s));
    if (loss) *loss = l;
    return JBGPU_OK;
}

int jbgpu_mlp_load_samples(jbgpu_mlp* h, const float* x, const float* t, int32_t n) {
    if (!h || n <= 0 || !x || !t) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "bad argument");
    MCK(cudaSetDevice(h->device));
    MCK(cudaStreamSynchronize(h->s));
    if (n > h->cap) {
        for (void* q : {(void*)h->X, (void*)h->T, (void*)h->idx}) if (q) cudaFree(q);
        h->X = h->T = nullptr;
        h->idx = nullptr;
        h->cap = 0;
        MCK(cudaMalloc(&h->X, sizeof(float) * (size_t)n * MLP_IN));
        MCK(cudaMalloc(&h->T, sizeof(float) * (size_t)n * MLP_OUT));
        MCK(cudaMalloc(&h->idx, sizeof(int) * (size_t)n));
        h->cap = n;
    }
    MCK(cudaMemcpy(h->X, x, sizeof(float) * (size_t)n * MLP_IN, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(h->T, t, sizeof(float) * (size_t)n * MLP_OUT, cudaMemcpyHostToDevice));
    h->n = n;
    return JBGPU_OK;
}

int jbgpu_mlp_train(jbgpu_mlp* h, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* loss_per_epoch) {
    if (!h || epochs <= 0 || batch < MLP_TILE || !(lr > 0.0f)) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "bad argument");
    if (h->n <= 0) return set_last_error(JBGPU_ERR_INVALID_ARGUMENT, "no samples loaded");
    MCK(cudaSetDevice(h->device));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    std::vector<int> perm(h->n);
    std::mt19937_64 rng(seed);
    for (int ep = 0; ep < epochs; ep++) {
        for (int i = 0; i < h->n; i++) perm[i] = i;
        std::shuffle(perm.begin(), perm.end(), rng);
        MCK(cudaMemcpyAsync(h->idx, perm.data(), sizeof(int) * (size_t)h->n, cudaMemcpyHostToDevice, h->s));
        MCK(cudaMemsetAsync(h->loss, 0, sizeof(float), h->s));
        int batches = 0;
        for (int first = 0; first < h->n; first += batch) {
            int count = std::min(batch, h->n - first);
            launch_train_batch(h, h->X, h->T, h->idx, first, count);
            ++h->adamStep;
            double t = (double)h->adamStep;
            float lr1 = (float)(lr / (1.0 - std::pow((double)b1, t)));
            float bc2 = (float)(1.0 / (1.0 - std::pow((double)b2, t)));
            k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, h->s>>>(h->p, h->g, h->m, h->v, lr1, bc2, b1, b2, eps);
            note_launch();
            int rc = mlp_repack(h);
            if (rc) return rc;
            ++batches;
        }
        MCK(cudaGetLastError());
        float l = 0.0f;
        MCK(cudaMemcpyAsync(&l, h->loss, sizeof(float), cudaMemcpyDeviceToHost, h->s));
        MCK(cudaStreamSynchronize(h->s));
        if (loss_per_epoch) loss_per_epoch[ep] = l / (float)batches;
    }
    return JBGPU_OK;
}

}  // extern "C"
