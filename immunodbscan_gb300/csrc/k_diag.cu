// k_diag.cu -- measurement helpers behind include/immunodbscan_gb300_diag.h.
//
// idb_diag_int_peak: the measured 32-bit integer-logic throughput of the GPU,
// the denominator of the distance kernel's roofline.  Every thread runs 8
// independent chains of lop3.b32 (the XOR/OR folds of the Hamming test) and
// add.u32 written in PTX, so the op count of the timed loop is known exactly.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/immunodbscan_gb300_diag.h"

namespace {

constexpr int kChains = 8;
constexpr int kOpsPerIter = kChains * 3;   // two lop3 + one add per chain

__global__ void __launch_bounds__(256) k_int_probe(uint32_t iters, uint32_t seed, uint32_t *out) {
    uint32_t a[kChains], b[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) {
        a[k] = seed ^ (threadIdx.x * 0x9E3779B9u + k);
        b[k] = seed + k * 0x85EBCA6Bu + blockIdx.x;
    }
    for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) {
            // a = (a ^ b) | i ; b = (b ^ a) & ~i-ish ; a += b
            asm volatile("lop3.b32 %0, %0, %1, %2, 0xBE;" : "+r"(a[k]) : "r"(b[k]), "r"(i));
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x6A;" : "+r"(b[k]) : "r"(a[k]), "r"(i));
            asm volatile("add.u32 %0, %0, %1;" : "+r"(a[k]) : "r"(b[k]));
        }
    }
    uint32_t r = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) r ^= a[k] ^ b[k];
    if (r == 0x12345678u) out[blockIdx.x] = r;   // keeps the chains alive
}

}  // namespace

extern "C" int idb_diag_int_peak(int device, double *gops_out, double *ms_out) {
    if (!gops_out) return 1;
    if (cudaSetDevice(device) != cudaSuccess) return 3;
    cudaGetLastError();
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_int_probe, 256, 0);
    const int grid = sms * (per_sm > 0 ? per_sm : 1);
    uint32_t *out = nullptr;
    if (cudaMalloc(&out, sizeof(uint32_t) * grid) != cudaSuccess) return 5;
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const uint32_t iters = 1u << 16;
    k_int_probe<<<grid, 256, 0, s>>>(1024, 1u, out);   // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0, s);
        k_int_probe<<<grid, 256, 0, s>>>(iters, 7u + rep, out);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    cudaFree(out);
    if (err != cudaSuccess) return 2;
    const double ops = (double)grid * 256.0 * iters * kOpsPerIter;
    *gops_out = ops / (best * 1e-3) / 1e9;
    if (ms_out) *ms_out = best;
    return 0;
}
