// csx_bench.cu — measurement kernels for bench.py's roofline (libcsx_bench.so).
//
// The screen is bound by 32-bit integer / FP32 issue, not by HBM or tensor
// cores, so its roofline denominators are measured here on the same GPU:
//   kind 0  integer ALU chain (shift, xor, add)        -> lane-ops / s
//   kind 1  IMAD chain                                 -> lane-ops / s
//   kind 2  FFMA chain                                 -> lane-ops / s
//   kind 3  splitmix64 outputs (full 64-bit mixer)     -> hashes / s
//   kind 4  DFMA chain (FP64 fused multiply-add)       -> lane-ops / s
// Each thread runs 8 independent chains so issue, not latency, is measured.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "../../include/csx_bench.h"

namespace {

constexpr int kChains = 8;

__global__ void alu_kernel(uint32_t *out, int iters, uint32_t seed) {
    uint32_t a[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = seed ^ (threadIdx.x * 0x9E3779B9u + j * 0x85EBCA6Bu);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kChains; ++j) a[j] = (a[j] ^ (a[j] >> 7)) + 0x7F4A7C15u;  // SHF, LOP3, IADD
    }
    uint32_t x = 0;
#pragma unroll
    for (int j = 0; j < kChains; ++j) x ^= a[j];
    if (x == 0x12345678u) out[0] = x;  // keeps the chains live
}

__global__ void imad_kernel(uint32_t *out, int iters, uint32_t seed) {
    uint32_t a[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = seed ^ (threadIdx.x * 0x9E3779B9u + j);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kChains; ++j) a[j] = a[j] * 0x2545F491u + 0x6C078965u;  // IMAD
    }
    uint32_t x = 0;
#pragma unroll
    for (int j = 0; j < kChains; ++j) x ^= a[j];
    if (x == 0x12345678u) out[0] = x;
}

__global__ void ffma_kernel(uint32_t *out, int iters, float seed) {
    float a[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = seed + threadIdx.x * 1e-7f + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kChains; ++j) a[j] = __fmaf_rn(a[j], 0.999999f, 1e-7f);  // FFMA
    }
    float x = 0;
#pragma unroll
    for (int j = 0; j < kChains; ++j) x += a[j];
    if (x == 1234.5f) out[0] = 1;
}

__global__ void dfma_kernel(uint32_t *out, int iters, double seed) {
    double a[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = seed + threadIdx.x * 1e-9 + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kChains; ++j) a[j] = fma(a[j], 0.9999999999, 1e-9);  // DFMA
    }
    double x = 0;
#pragma unroll
    for (int j = 0; j < kChains; ++j) x += a[j];
    if (x == 1234.5) out[0] = 1;
}

__global__ void hash_kernel(uint32_t *out, int iters, uint64_t seed) {
    uint64_t s[kChains];
    uint64_t acc = 0;
#pragma unroll
    for (int j = 0; j < kChains; ++j) s[j] = seed + (threadIdx.x + blockIdx.x * blockDim.x) * 977ull + j;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kChains; ++j) {
            s[j] += 0x9E3779B97F4A7C15ull;
            uint64_t z = s[j];
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            acc += z ^ (z >> 31);
        }
    }
    if (acc == 0x123456789ull) out[0] = 1;
}

}  // namespace

extern "C" int csx_bench_issue_rate(int kind, double *per_second) {
    if (!per_second || kind < 0 || kind > 4) return -3;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -8;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint32_t *out = nullptr;
    if (cudaMalloc(&out, 16) != cudaSuccess) return -9;
    const int threads = 256, blocks = sms * 8;
    const int iters = kind >= 3 ? 2000 : 20000;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(a);
        switch (kind) {
            case 0: alu_kernel<<<blocks, threads>>>(out, iters, rep); break;
            case 1: imad_kernel<<<blocks, threads>>>(out, iters, rep); break;
            case 2: ffma_kernel<<<blocks, threads>>>(out, iters, 1.0f + rep); break;
            case 4: dfma_kernel<<<blocks, threads>>>(out, iters, 1.0 + rep); break;
            default: hash_kernel<<<blocks, threads>>>(out, iters, rep); break;
        }
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
    }
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "csx_bench: %s\n", cudaGetErrorString(e));
        return -7;
    }
    const double ops_per_iter = kind == 0 ? 3.0 : 1.0;  // lane-ops (kinds 0-2, 4) or hashes (3)
    *per_second = static_cast<double>(blocks) * threads * iters * kChains * ops_per_iter / (best * 1e-3);
    return 0;
}
