// k_mlp.cu -- the learned work predictor of the distance scheduler.
//
// A 16 -> 64 -> 64 -> 1 multilayer perceptron (ReLU) predicts log2 of the
// device cycles a bin pair will take, from features of the pair: entry counts,
// pair count, length gap, lengths, eps, unit count and the static class.  The persistent distance kernel hands out work units heavy-first;
// with the learned schedule, "heavy" is the prediction instead of the pair count.
// The method's answer never depends on the schedule.
//
// Training (FP32): a block takes a tile of 64 samples, keeps the activations in
// shared memory and forms the weight gradients as small matrix products over the
// tile; an Adam step updates the weights.  Inference (BF16 weights and
// activations, FP32 accumulation) runs on the bin-pair list of a call, before
// the schedule is built.
//
// No counterpart in the reference, which schedules nothing (one block per pair
// over the full n_u x n_u grid, cuda/PSDBSCAN.hcu:1115-1167).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "idb_internal.cuh"

namespace idb {

// parameter block layout (floats): W1[16][64] b1[64] W2[64][64] b2[64] w3[64] b3
constexpr int kIn = kMlpIn, kH = kMlpHidden;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kH;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kH;
static_assert(kOffB3 + 1 == kMlpParams, "parameter layout");

namespace {

constexpr int kThreads = 128;
constexpr uint32_t kLearnMinPairs = 4096;   // smaller bin pairs skip the network
constexpr float kLightCyclesPerPair = 32.0f;

// Features of one bin pair (also used by the host to build training sets).
__device__ void binpair_features(const BinPair &P, float *f) {
    const float na = (float)P.a_n, nb = (float)P.b_n;
    const float pairs = P.same ? 0.5f * na * (na - 1.0f) : na * nb;
    f[0] = log2f(1.0f + na);
    f[1] = log2f(1.0f + (P.same ? na : nb));
    f[2] = P.same ? 1.0f : 0.0f;
    f[3] = (float)(P.lb - P.la);
    f[4] = (float)P.la * (1.0f / 32.0f);
    f[5] = (float)P.eps;
    f[6] = log2f(1.0f + pairs);
    f[7] = f[0] * f[0] * (1.0f / 64.0f);
    f[8] = (float)(P.la + P.lb) * (1.0f / 64.0f);
    f[9] = log2f(1.0f + (float)P.ncx);
    f[10] = (float)P.cls;
    f[11] = f[0] * f[1] * (1.0f / 16.0f);
    f[12] = (float)P.lb * (1.0f / 32.0f);
    f[13] = P.eps > 0 ? (float)(P.lb - P.la) / (float)P.eps : 0.0f;
    f[14] = log2f(1.0f + fminf(na, nb));
    f[15] = 1.0f;
}

__global__ void k_features(const Counters *__restrict__ ctr, const BinPair *__restrict__ bp,
                           float *__restrict__ feats) {
    const uint32_t n = ctr->n_binpairs;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float f[kIn];
        binpair_features(bp[i], f);
#pragma unroll
        for (int k = 0; k < kIn; ++k) feats[(size_t)i * kIn + k] = f[k];
    }
}

// Bin pairs below kLearnMinPairs skip the network: their cost is their pair
// count times kLightCyclesPerPair (a middle value of the logged cycles per
// pair), which keeps them after the heavy ones and in the static order among
// themselves; the others are listed for the network.
__global__ void k_mlp_select(Counters *ctr, const BinPair *__restrict__ bp,
                             float *__restrict__ pred, uint32_t *__restrict__ heavy) {
    const uint32_t n = ctr->n_binpairs;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < n; i0 += stride) {
        const uint32_t i = i0 + (threadIdx.x & 31);
        const bool big = i < n && bp[i].cost_lo >= kLearnMinPairs;
        if (i < n && !big) pred[i] = fmaxf(1.0f, (float)bp[i].cost_lo * kLightCyclesPerPair);
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, big);
        uint32_t b0 = 0;
        if ((threadIdx.x & 31) == 0 && m) b0 = atomicAdd(&ctr->n_heavy, (uint32_t)__popc(m));
        b0 = __shfl_sync(0xFFFFFFFFu, b0, 0);
        if (big) heavy[b0 + __popc(m & ((1u << (threadIdx.x & 31)) - 1u))] = i;
    }
}

// BF16 forward pass of one sample by one warp (weights in shared memory):
// inputs and hidden activations rounded to BF16, products accumulated in FP32.
// Lane j computes hidden units j and j+32 of both layers (each a dot product
// in ascending input order, starting from the bias); the output layer sums the
// second layer in ascending unit order.  Every lane returns the predicted log2
// cycles.  A warp per sample keeps the 5k multiply-adds of a sample spread
// over 32 lanes instead of one long chain.
__device__ __forceinline__ float mlp_forward_bf16_warp(const __nv_bfloat16 *w, const float (&f)[kIn],
                                                       float *s_h2, int lane) {
    const int j0 = lane, j1 = lane + 32;
    float a0 = __bfloat162float(w[kOffB1 + j0]), a1 = __bfloat162float(w[kOffB1 + j1]);
#pragma unroll
    for (int k = 0; k < kIn; ++k) {
        const float x = __bfloat162float(__float2bfloat16(f[k]));
        a0 = fmaf(x, __bfloat162float(w[kOffW1 + k * kH + j0]), a0);
        a1 = fmaf(x, __bfloat162float(w[kOffW1 + k * kH + j1]), a1);
    }
    const float h1a = __bfloat162float(__float2bfloat16(fmaxf(a0, 0.0f)));
    const float h1b = __bfloat162float(__float2bfloat16(fmaxf(a1, 0.0f)));
    float c0 = __bfloat162float(w[kOffB2 + j0]), c1 = __bfloat162float(w[kOffB2 + j1]);
#pragma unroll 8
    for (int k = 0; k < kH; ++k) {
        const float hk = __shfl_sync(0xFFFFFFFFu, k < 32 ? h1a : h1b, k & 31);
        c0 = fmaf(hk, __bfloat162float(w[kOffW2 + k * kH + j0]), c0);
        c1 = fmaf(hk, __bfloat162float(w[kOffW2 + k * kH + j1]), c1);
    }
    s_h2[j0] = __bfloat162float(__float2bfloat16(fmaxf(c0, 0.0f)));
    s_h2[j1] = __bfloat162float(__float2bfloat16(fmaxf(c1, 0.0f)));
    __syncwarp();
    float y = __bfloat162float(w[kOffB3]);
    for (int j = 0; j < kH; ++j) y = fmaf(s_h2[j], __bfloat162float(w[kOffW3 + j]), y);
    __syncwarp();
    return y;
}

// BF16 inference over the listed bin pairs, a warp per bin pair:
// pred[i] = 2^mlp(features)
__global__ void __launch_bounds__(kThreads)
k_mlp_predict_bf16(const Counters *__restrict__ ctr, const BinPair *__restrict__ bp,
                   const uint32_t *__restrict__ heavy, const __nv_bfloat16 *__restrict__ wq,
                   float *__restrict__ pred) {
    __shared__ __nv_bfloat16 w[kMlpParams];
    __shared__ float s_h2[kThreads / 32][kH];
    const uint32_t n = ctr->n_heavy;
    const uint32_t warps = gridDim.x * (kThreads / 32);
    if (blockIdx.x * (kThreads / 32) >= n) return;   // no sample for this block
    for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) w[k] = wq[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t k0 = blockIdx.x * (kThreads / 32) + wid; k0 < n; k0 += warps) {
        const uint32_t i = heavy[k0];
        float f[kIn];
        binpair_features(bp[i], f);
        const float y = mlp_forward_bf16_warp(w, f, s_h2[wid], lane);
        if (lane == 0) pred[i] = exp2f(fminf(y, 60.0f));
    }
}

// The same forward pass on given feature rows (log2 cycles out), for checking
// the inference against a CPU forward pass.
__global__ void __launch_bounds__(kThreads)
k_mlp_forward_rows(const float *__restrict__ X, uint32_t n, const __nv_bfloat16 *__restrict__ wq,
                   float *__restrict__ y) {
    __shared__ __nv_bfloat16 w[kMlpParams];
    __shared__ float s_h2[kThreads / 32][kH];
    for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) w[k] = wq[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t warps = gridDim.x * (kThreads / 32);
    for (uint32_t i = blockIdx.x * (kThreads / 32) + wid; i < n; i += warps) {
        float f[kIn];
#pragma unroll
        for (int k = 0; k < kIn; ++k) f[k] = X[(size_t)i * kIn + k];
        const float v = mlp_forward_bf16_warp(w, f, s_h2[wid], lane);
        if (lane == 0) y[i] = v;
    }
}

// FP32 forward + backward.  A block takes a tile of 64 samples; activations
// live in shared memory and the weight gradients are small matrix products over
// the tile (dW2 = H1^T D2, dW1 = X^T D1), added to `grad` with one atomic per
// parameter per tile.  loss += sum of squared errors; `scale` turns the sum into
// a mean (1/n).
constexpr int kTile = 64;
constexpr int kGradThreads = 256;

__global__ void __launch_bounds__(kGradThreads)
k_mlp_grad(const float *__restrict__ X, const float *__restrict__ T, uint32_t n,
           const float *__restrict__ p, float scale, float *__restrict__ grad,
           float *__restrict__ loss) {
    extern __shared__ float sh[];
    float *w = sh;                              // kMlpParams
    float *x = w + kMlpParams;                  // [kTile][kIn]
    float *z1 = x + kTile * kIn;                // [kTile][kH]  pre-activation of layer 1
    float *z2 = z1 + kTile * kH;                // [kTile][kH]  pre-activation of layer 2, then D2
    float *dy = z2 + kTile * kH;                // [kTile]
    float *d1 = dy + kTile;                     // [kTile][kH]
    const int t = threadIdx.x;
    for (int k = t; k < kMlpParams; k += blockDim.x) w[k] = p[k];
    __syncthreads();
    const uint32_t ntiles = (n + kTile - 1) / kTile;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t s0 = tile * kTile;
        const int ns = (int)min((uint32_t)kTile, n - s0);
        for (int k = t; k < kTile * kIn; k += blockDim.x) {
            const int si = k / kIn;
            x[k] = si < ns ? X[(size_t)(s0 + si) * kIn + (k % kIn)] : 0.0f;
        }
        __syncthreads();
        // layer 1: 4 threads per sample, 16 hidden units each
        const int si = t >> 2, j0 = (t & 3) * 16;
        for (int j = j0; j < j0 + 16; ++j) {
            float acc = w[kOffB1 + j];
#pragma unroll
            for (int k = 0; k < kIn; ++k) acc = fmaf(x[si * kIn + k], w[kOffW1 + k * kH + j], acc);
            z1[si * kH + j] = acc;
        }
        __syncthreads();
        float ypart = 0.0f;
        for (int j = j0; j < j0 + 16; ++j) {
            float acc = w[kOffB2 + j];
            for (int k = 0; k < kH; ++k) acc = fmaf(fmaxf(z1[si * kH + k], 0.0f), w[kOffW2 + k * kH + j], acc);
            z2[si * kH + j] = acc;
            ypart = fmaf(fmaxf(acc, 0.0f), w[kOffW3 + j], ypart);
        }
        ypart += __shfl_xor_sync(0xFFFFFFFFu, ypart, 1);
        ypart += __shfl_xor_sync(0xFFFFFFFFu, ypart, 2);
        if ((t & 3) == 0) {
            float d = 0.0f;
            if (si < ns) {
                const float err = ypart + w[kOffB3] - T[s0 + si];
                atomicAdd(loss, err * err);
                d = 2.0f * err * scale;
            }
            dy[si] = d;
        }
        __syncthreads();
        // output layer gradients and D2 = dy * w3 * relu'(z2)
        if (t < kH) {
            float gw = 0.0f;
            for (int s = 0; s < kTile; ++s) gw = fmaf(dy[s], fmaxf(z2[s * kH + t], 0.0f), gw);
            atomicAdd(&grad[kOffW3 + t], gw);
        } else if (t == kH) {
            float gb = 0.0f;
            for (int s = 0; s < kTile; ++s) gb += dy[s];
            atomicAdd(&grad[kOffB3], gb);
        }
        __syncthreads();
        for (int k = t; k < kTile * kH; k += blockDim.x) {
            const int s = k / kH, j = k % kH;
            z2[k] = z2[k] > 0.0f ? dy[s] * w[kOffW3 + j] : 0.0f;
        }
        __syncthreads();
        // dW2[k][j] = sum_s relu(z1[s][k]) D2[s][j]; db2[j] = sum_s D2[s][j]
        for (int e = t; e < kH * kH; e += blockDim.x) {
            const int k = e / kH, j = e % kH;
            float acc = 0.0f;
            for (int s = 0; s < kTile; ++s) acc = fmaf(fmaxf(z1[s * kH + k], 0.0f), z2[s * kH + j], acc);
            if (acc != 0.0f) atomicAdd(&grad[kOffW2 + e], acc);
        }
        if (t < kH) {
            float acc = 0.0f;
            for (int s = 0; s < kTile; ++s) acc += z2[s * kH + t];
            atomicAdd(&grad[kOffB2 + t], acc);
        }
        // D1[s][k] = relu'(z1[s][k]) * sum_j D2[s][j] W2[k][j]
        for (int e = t; e < kTile * kH; e += blockDim.x) {
            const int s = e / kH, k = e % kH;
            float acc = 0.0f;
            if (z1[e] > 0.0f)
                for (int j = 0; j < kH; ++j) acc = fmaf(z2[s * kH + j], w[kOffW2 + k * kH + j], acc);
            d1[e] = acc;
        }
        __syncthreads();
        // dW1[k][j] = sum_s x[s][k] D1[s][j]; db1[j] = sum_s D1[s][j]
        for (int e = t; e < kIn * kH; e += blockDim.x) {
            const int k = e / kH, j = e % kH;
            float acc = 0.0f;
            for (int s = 0; s < kTile; ++s) acc = fmaf(x[s * kIn + k], d1[s * kH + j], acc);
            if (acc != 0.0f) atomicAdd(&grad[kOffW1 + e], acc);
        }
        if (t < kH) {
            float acc = 0.0f;
            for (int s = 0; s < kTile; ++s) acc += d1[s * kH + t];
            atomicAdd(&grad[kOffB1 + t], acc);
        }
        __syncthreads();
    }
}

constexpr size_t kGradSmem =
    sizeof(float) * (kMlpParams + kTile * kIn + 3 * kTile * kH + kTile);

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ grad, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kMlpParams) return;
    const float gk = grad[k];
    const float mk = b1 * m[k] + (1.0f - b1) * gk;
    const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

__global__ void k_to_bf16(const float *__restrict__ p, __nv_bfloat16 *__restrict__ q) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < kMlpParams) q[k] = __float2bfloat16(p[k]);
}

}  // namespace

void launch_features(const Buffers &B, uint32_t cap, float *feats, cudaStream_t s) {
    const int grid = (int)std::min<uint64_t>((cap + kThreads - 1) / kThreads, (uint64_t)sm_count() * 8);
    k_features<<<grid > 0 ? grid : 1, kThreads, 0, s>>>(B.ctr, B.bp_sorted, feats);
}

// The heavy list lives in bp_small, which the schedule fills only afterwards.
void launch_mlp_predict(const Buffers &B, uint32_t cap, const void *wq_bf16, cudaStream_t s) {
    cudaMemsetAsync(&B.ctr->n_heavy, 0, sizeof(uint32_t), s);
    const int gsel = (int)std::min<uint64_t>((cap + 255) / 256, (uint64_t)sm_count() * 8);
    k_mlp_select<<<gsel > 0 ? gsel : 1, 256, 0, s>>>(B.ctr, B.bp, B.pred, B.bp_small);
    constexpr uint32_t kWarpsPerBlock = kThreads / 32;   // a warp per listed bin pair
    const int grid = (int)std::min<uint64_t>((cap + kWarpsPerBlock - 1) / kWarpsPerBlock,
                                             (uint64_t)sm_count() * 8);
    k_mlp_predict_bf16<<<grid > 0 ? grid : 1, kThreads, 0, s>>>(
        B.ctr, B.bp, B.bp_small, static_cast<const __nv_bfloat16 *>(wq_bf16), B.pred);
}

void launch_mlp_grad(const float *X, const float *T, uint32_t n, const float *p, float scale,
                     float *grad, float *loss, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem);
        attr = true;
    }
    const int grid = (int)std::min<uint64_t>((n + kTile - 1) / kTile, (uint64_t)sm_count() * 2);
    k_mlp_grad<<<grid > 0 ? grid : 1, kGradThreads, kGradSmem, s>>>(X, T, n, p, scale, grad, loss);
}

void launch_adam(float *p, const float *grad, float *m, float *v, float lr, int step,
                 cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    k_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(p, grad, m, v, lr, b1, b2, 1e-8f, c1, c2);
}

void launch_mlp_forward_rows(const float *X, uint32_t n, const void *wq_bf16, float *y,
                             cudaStream_t s) {
    const int grid = (int)std::min<uint64_t>((n + kThreads / 32 - 1) / (kThreads / 32),
                                             (uint64_t)sm_count() * 8);
    k_mlp_forward_rows<<<grid > 0 ? grid : 1, kThreads, 0, s>>>(
        X, n, static_cast<const __nv_bfloat16 *>(wq_bf16), y);
}

void launch_to_bf16(const float *p, void *q, cudaStream_t s) {
    k_to_bf16<<<(kMlpParams + 255) / 256, 256, 0, s>>>(p, static_cast<__nv_bfloat16 *>(q));
}

}  // namespace idb
