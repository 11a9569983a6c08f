// Kernels of the learned tracklet pre-filter: weight packing, tensor-core
// scoring of feature rows, and the training step (forward + backward on the
// CUDA cores with the inference path's BF16 roundings, then Adam).
#include <cstdio>

#include "sdl_mlp.h"

namespace sdlg {

namespace {

// FP32 parameters -> packed BF16 tiles [W1 b1], W2, b2 and the FP32 tail
// (BF16-rounded w3, b3, threshold)
__global__ void k_mlp_pack(const float* __restrict__ p, unsigned char* __restrict__ pack, float thr) {
    for (int e = threadIdx.x; e < kMlpHid * kMlpK1; e += blockDim.x) {
        const int n = e / kMlpK1, k = e % kMlpK1;
        const float w = k < kMlpIn ? p[kMlpW1 + n * kMlpIn + k] : (k == kMlpIn ? p[kMlpB1 + n] : 0.f);
        *reinterpret_cast<uint16_t*>(pack + kPackW1 + cm_offset(n, k, 2)) = bf16_bits(w);
    }
    for (int e = threadIdx.x; e < kMlpHid * kMlpK2; e += blockDim.x) {
        const int n = e / kMlpK2, k = e % kMlpK2;
        *reinterpret_cast<uint16_t*>(pack + kPackW2 + cm_offset(n, k, 8)) = bf16_bits(p[kMlpW2 + n * kMlpHid + k]);
    }
    for (int e = threadIdx.x; e < kMlpHid * 16; e += blockDim.x) {
        const int n = e / 16, k = e % 16;
        *reinterpret_cast<uint16_t*>(pack + kPackB2 + cm_offset(n, k, 2)) = k == 0 ? bf16_bits(p[kMlpB2 + n]) : (uint16_t)0;
    }
    for (int n = threadIdx.x; n < kMlpHid; n += blockDim.x) reinterpret_cast<float*>(pack + kPackW3)[n] = bf16_round(p[kMlpW3 + n]);
    if (threadIdx.x == 0) {
        float* tail = reinterpret_cast<float*>(pack + kPackB3);
        tail[0] = p[kMlpB3];
        tail[1] = thr;
        tail[2] = 0.f;
        tail[3] = 0.f;
    }
}

// logits of n feature rows (row-major n x 12), one 128-row tile per step
__global__ void __launch_bounds__(kMlpTile) k_mlp_score(const float* __restrict__ x, int64_t n,
                                                        const unsigned char* __restrict__ pack, float* __restrict__ logits,
                                                        unsigned int* __restrict__ status) {
    __shared__ MlpSmem sm;
    mlp_setup(sm, pack);
    MlpThread st;
    const int64_t ntile = (n + kMlpTile - 1) / kMlpTile;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int64_t r = tile * kMlpTile + threadIdx.x;
        float f[kMlpIn];
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) f[k] = r < n ? x[r * kMlpIn + k] : 0.f;
        const float z = mlp_tile(sm, f, st);
        if (r < n) logits[r] = z;
    }
    if (st.abort && threadIdx.x == 0) atomicOr(status, 1u);
    mlp_teardown(sm, st);
}

// ------------------------------------------------------------------ training
constexpr int kTrainRows = 128;   // samples per block
constexpr int kLd = kMlpHid + 1;  // padded row stride of the per-sample hidden arrays

struct TrainSmem {
    float w[kMlpParams];          // BF16-rounded weights and biases (b3 FP32)
    float x[kTrainRows][kMlpIn];  // BF16-rounded features
    float h1[kTrainRows][kLd];    // BF16-rounded ReLU outputs of layer 1
    float h2[kTrainRows][kLd];    // layer-2 ReLU outputs, then dLoss/da2
    float d1[kTrainRows][kLd];    // dLoss/da1
    float dz[kTrainRows];
    float loss[kTrainRows / 32];
};

__device__ __forceinline__ float sigmoid_f(float z) {
    if (z >= 0.f) return 1.f / (1.f + expf(-z));
    const float e = expf(z);
    return e / (1.f + e);
}
__device__ __forceinline__ float softplus_f(float z) { return fmaxf(z, 0.f) + log1pf(expf(-fabsf(z))); }

// Forward and backward over `count` samples (ids order[start + i], or
// start + i when order is null); adds inv_norm * sum_i w_i dLoss_i/dparam
// into grad and the weighted loss sum into loss.  Weighted logistic loss:
// w_i * (softplus(z_i) - y_i z_i).  The BF16 roundings of the forward pass
// are treated as the identity in the backward pass.
__global__ void __launch_bounds__(kTrainRows) k_mlp_fwd_bwd(const float* __restrict__ X, const float* __restrict__ Y,
                                                            const float* __restrict__ Wt, const int32_t* __restrict__ order,
                                                            int64_t start, int64_t count, float pos_weight, float inv_norm,
                                                            const float* __restrict__ params, float* __restrict__ grad,
                                                            double* __restrict__ loss) {
    extern __shared__ __align__(16) unsigned char smraw[];
    TrainSmem& sm = *reinterpret_cast<TrainSmem*>(smraw);
    const int t = threadIdx.x;
    for (int e = t; e < kMlpParams; e += blockDim.x) {
        const float v = params[e];
        sm.w[e] = e == kMlpB3 ? v : bf16_round(v);
    }
    const int64_t i = (int64_t)blockIdx.x * kTrainRows + t;
    const bool valid = i < count;
    int64_t id = 0;
    float y = 0.f, wt = 0.f;
    if (valid) {
        id = order ? (int64_t)order[start + i] : start + i;
        y = Y[id];
        wt = Wt ? Wt[id] : (y > 0.5f ? pos_weight : 1.f);
    }
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) sm.x[t][k] = valid ? bf16_round(X[id * kMlpIn + k]) : 0.f;
    __syncthreads();
    // forward (thread = sample)
    const float* W1 = sm.w + kMlpW1;
    const float* B1 = sm.w + kMlpB1;
    const float* W2 = sm.w + kMlpW2;
    const float* B2 = sm.w + kMlpB2;
    const float* W3 = sm.w + kMlpW3;
    for (int n = 0; n < kMlpHid; ++n) {
        float a = 0.f;
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) a = __fmaf_rn(W1[n * kMlpIn + k], sm.x[t][k], a);
        sm.h1[t][n] = bf16_round(fmaxf(__fadd_rn(a, B1[n]), 0.f));
    }
    float z = sm.w[kMlpB3];
    for (int n = 0; n < kMlpHid; ++n) {
        float a = 0.f;
#pragma unroll 16
        for (int j = 0; j < kMlpHid; ++j) a = __fmaf_rn(W2[n * kMlpHid + j], sm.h1[t][j], a);
        const float h = fmaxf(__fadd_rn(a, B2[n]), 0.f);
        sm.h2[t][n] = h;
        z = __fmaf_rn(W3[n], h, z);
    }
    const float l = valid ? wt * (softplus_f(z) - y * z) : 0.f;
    const float dz = valid ? wt * (sigmoid_f(z) - y) * inv_norm : 0.f;
    sm.dz[t] = dz;
    float ls = l;
    for (int o = 16; o > 0; o >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, o);
    if ((t & 31) == 0) sm.loss[t >> 5] = ls;
    __syncthreads();
    // gw3, gb3: reduce over samples (threads 0..63 own one unit each)
    if (t < kMlpHid) {
        float g = 0.f;
        for (int m = 0; m < kTrainRows; ++m) g = __fmaf_rn(sm.dz[m], sm.h2[m][t], g);
        atomicAdd(grad + kMlpW3 + t, g);
    } else if (t == kMlpHid) {
        float g = 0.f;
        for (int m = 0; m < kTrainRows; ++m) g += sm.dz[m];
        atomicAdd(grad + kMlpB3, g);
        double s = 0.0;
        for (int w = 0; w < kTrainRows / 32; ++w) s += (double)sm.loss[w];
        atomicAdd(loss, s);
    }
    __syncthreads();
    // dLoss/da2 (own sample), in place of h2
    for (int n = 0; n < kMlpHid; ++n) sm.h2[t][n] = sm.h2[t][n] > 0.f ? dz * W3[n] : 0.f;
    // dLoss/da1 (own sample)
    for (int j = 0; j < kMlpHid; ++j) {
        float a = 0.f;
        if (sm.h1[t][j] > 0.f) {
#pragma unroll 16
            for (int n = 0; n < kMlpHid; ++n) a = __fmaf_rn(sm.h2[t][n], W2[n * kMlpHid + j], a);
        }
        sm.d1[t][j] = a;
    }
    __syncthreads();
    // gW2[n][j] = sum_m d2[m][n] h1[m][j]; gb2
    for (int e = t; e < kMlpHid * kMlpHid; e += blockDim.x) {
        const int n = e / kMlpHid, j = e % kMlpHid;
        float g = 0.f;
        for (int m = 0; m < kTrainRows; ++m) g = __fmaf_rn(sm.h2[m][n], sm.h1[m][j], g);
        atomicAdd(grad + kMlpW2 + e, g);
    }
    // gW1[n][k] = sum_m d1[m][n] x[m][k]; gb1, gb2
    for (int e = t; e < kMlpHid * kMlpIn; e += blockDim.x) {
        const int n = e / kMlpIn, k = e % kMlpIn;
        float g = 0.f;
        for (int m = 0; m < kTrainRows; ++m) g = __fmaf_rn(sm.d1[m][n], sm.x[m][k], g);
        atomicAdd(grad + kMlpW1 + e, g);
    }
    if (t < kMlpHid) {
        float g1 = 0.f, g2 = 0.f;
        for (int m = 0; m < kTrainRows; ++m) {
            g1 += sm.d1[m][t];
            g2 += sm.h2[m][t];
        }
        atomicAdd(grad + kMlpB1 + t, g1);
        atomicAdd(grad + kMlpB2 + t, g2);
    }
}

// Adam step on the FP32 master parameters; clears the gradient
__global__ void k_mlp_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                           float lr, float c1, float c2) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kMlpParams; e += gridDim.x * blockDim.x) {
        const float gr = g[e];
        const float mm = b1 * m[e] + (1.f - b1) * gr;
        const float vv = b2 * v[e] + (1.f - b2) * gr * gr;
        m[e] = mm;
        v[e] = vv;
        p[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
        g[e] = 0.f;
    }
}

}  // namespace

size_t mlp_train_smem() { return sizeof(TrainSmem); }

void launch_mlp_pack(const float* params, unsigned char* pack, float thr, cudaStream_t s) {
    k_mlp_pack<<<1, 256, 0, s>>>(params, pack, thr);
}

void launch_mlp_score(const float* x, int64_t n, const unsigned char* pack, float* logits, unsigned int* status, int n_sm,
                      cudaStream_t s) {
    if (n <= 0) return;
    const int64_t ntile = (n + kMlpTile - 1) / kMlpTile;
    const int64_t grid = ntile < (int64_t)n_sm * 4 ? ntile : (int64_t)n_sm * 4;
    k_mlp_score<<<(unsigned)grid, kMlpTile, 0, s>>>(x, n, pack, logits, status);
}

cudaError_t launch_mlp_fwd_bwd(const float* X, const float* Y, const float* W, const int32_t* order, int64_t start,
                               int64_t count, float pos_weight, float inv_norm, const float* params, float* grad,
                               double* loss, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_mlp_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((count + kTrainRows - 1) / kTrainRows);
    k_mlp_fwd_bwd<<<grid, kTrainRows, sizeof(TrainSmem), s>>>(X, Y, W, order, start, count, pos_weight, inv_norm, params,
                                                               grad, loss);
    return cudaGetLastError();
}

void launch_mlp_adam(float* p, float* g, float* m, float* v, float lr, float c1, float c2, cudaStream_t s) {
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(p, g, m, v, lr, c1, c2);
}

}  // namespace sdlg
