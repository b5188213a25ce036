// The quadratic surrogate as a differentiable function: forward, backward,
// the ridge refit's normal equations, an FP64 Cholesky solve and a
// gradient-ascent mutation step (include/csx_surrogate.h).
//
// Reference: brain/evolve.py:211-220 (features: [1 | genes | g_i g_j, j <= i
// < 16]) and :250-268 (refit_surrogate: numpy FP64 normal equations and
// solve); src/screen.zig:97-112 (the screen's score of the same features).
//
// Work sizes are small next to the screen: a refit table of 400,000 rows of
// 16 genes is 25.6 MB. The normal equations are FP64 multiply-adds
// (nf(nf+1)/2 per row) and run on the FP64 pipe; everything else is a few
// hundred FP32 FMAs per row.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "csx_screen.h"
#include "csx_surrogate.h"

namespace {

constexpr int kQuadGenes = 16;
constexpr int kNQuad = kQuadGenes * (kQuadGenes + 1) / 2;  // 136
constexpr int kMaxLin = 29;
constexpr int kMinFeat = 1 + kQuadGenes + kNQuad;  // 153
constexpr int kMaxFeat = 1 + kMaxLin + kNQuad;     // 166
constexpr int kRowThreads = 256;                   // rows per tile in the row kernels
constexpr int kPartBlocks = 152;                   // fixed: the reductions' summation order never changes
constexpr int kGramRows = 32;                      // rows per Φ tile in the normal equations
constexpr int kGramBlk = 4;                        // each thread owns a 4×4 block of ΦᵀΦ
constexpr int kGramNb = (kMaxFeat + kGramBlk - 1) / kGramBlk;  // 42 block rows at most
constexpr int kGramPairs = kGramNb * (kGramNb + 1) / 2;        // 903 lower-triangle blocks at most
constexpr int kGramFeatPad = kGramNb * kGramBlk;               // 168
constexpr int kSolveThreads = 1024;

__host__ __device__ constexpr int tri(int i) { return i * (i + 1) / 2; }

// Coefficients as the row kernels read them: linear terms padded with zeros to
// 29, quadratic terms packed (i, j <= i).
struct CoefF {
    float c0;
    float lin[kMaxLin];
    float q[kNQuad];
};

template <int P>
__device__ __forceinline__ float in_prec(float x) {
    if constexpr (P == CSX_SG_BF16) return __bfloat162float(__float2bfloat16_rn(x));
    return x;
}

template <int P>
__device__ void load_coef(CoefF &s, const float *coef, int ng) {
    for (int i = threadIdx.x; i < 1 + kMaxLin + kNQuad; i += blockDim.x) {
        float v;
        if (i == 0) {
            v = coef[0];
        } else if (i <= kMaxLin) {
            v = (i <= ng) ? coef[i] : 0.0f;
        } else {
            v = coef[1 + ng + (i - 1 - kMaxLin)];
        }
        reinterpret_cast<float *>(&s)[i] = in_prec<P>(v);
    }
}

// Stage rows [r0, r0 + kRowThreads) of the gene table into shared memory
// (coalesced), row stride `st` (odd, so a thread-per-row read is conflict free).
__device__ void stage_rows(float *tile, const float *genes, int64_t n, int ldg, int ng, int st, int64_t r0) {
    const int64_t rows = (n - r0 < kRowThreads) ? (n - r0) : kRowThreads;
    const int total = static_cast<int>(rows) * ng;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int r = idx / ng, k = idx - r * ng;
        tile[r * st + k] = genes[(r0 + r) * static_cast<int64_t>(ldg) + k];
    }
}

template <int P>
__device__ __forceinline__ void read_row(float (&g)[kMaxLin], const float *tile, int st, int ng) {
#pragma unroll
    for (int k = 0; k < kMaxLin; ++k) g[k] = (k < ng) ? in_prec<P>(tile[threadIdx.x * st + k]) : 0.0f;
}

__device__ __forceinline__ float score_f32(const CoefF &c, const float (&g)[kMaxLin]) {
    float s = c.c0;
#pragma unroll
    for (int k = 0; k < kMaxLin; ++k) s = __fmaf_rn(c.lin[k], g[k], s);
#pragma unroll
    for (int i = 0; i < kQuadGenes; ++i) {
        float t = 0.0f;
#pragma unroll
        for (int j = 0; j <= i; ++j) t = __fmaf_rn(c.q[tri(i) + j], g[j], t);
        s = __fmaf_rn(t, g[i], s);
    }
    return s;
}

// ∂score/∂g_k = lin_k + Σ_{j<=k} q_kj g_j + Σ_{i>=k} q_ik g_i (k < 16).
__device__ __forceinline__ void grad_f32(const CoefF &c, const float (&g)[kMaxLin], float (&d)[kMaxLin]) {
#pragma unroll
    for (int k = 0; k < kMaxLin; ++k) d[k] = c.lin[k];
#pragma unroll
    for (int i = 0; i < kQuadGenes; ++i) {
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            const float q = c.q[tri(i) + j];
            d[i] = __fmaf_rn(q, g[j], d[i]);
            d[j] = __fmaf_rn(q, g[i], d[j]);
        }
    }
}

__host__ __device__ inline int stride_for(int ng) { return ((ng + 1) & 1) ? ng + 1 : ng + 2; }  // odd, >= ng + 1

template <int P>
__global__ void __launch_bounds__(kRowThreads) sg_forward_kernel(const float *__restrict__ coef, int ng,
                                                                 const float *__restrict__ genes, int64_t n,
                                                                 int ldg, float *__restrict__ score) {
    __shared__ CoefF c;
    extern __shared__ float tile[];
    const int st = stride_for(ng);
    load_coef<P>(c, coef, ng);
    for (int64_t r0 = static_cast<int64_t>(blockIdx.x) * kRowThreads; r0 < n;
         r0 += static_cast<int64_t>(gridDim.x) * kRowThreads) {
        __syncthreads();
        stage_rows(tile, genes, n, ldg, ng, st, r0);
        __syncthreads();
        if (r0 + threadIdx.x < n) {
            float g[kMaxLin];
            read_row<P>(g, tile, st, ng);
            score[r0 + threadIdx.x] = score_f32(c, g);
        }
    }
}

__global__ void __launch_bounds__(kRowThreads) sg_forward_f64_kernel(const double *__restrict__ coef, int ng,
                                                                     const float *__restrict__ genes, int64_t n,
                                                                     int ldg, double *__restrict__ score) {
    __shared__ double lin[kMaxLin], q[kNQuad], c0;
    extern __shared__ float tile[];
    const int st = stride_for(ng);
    for (int i = threadIdx.x; i < 1 + kMaxLin + kNQuad; i += blockDim.x) {
        if (i == 0) c0 = coef[0];
        else if (i <= kMaxLin) lin[i - 1] = (i <= ng) ? coef[i] : 0.0;
        else q[i - 1 - kMaxLin] = coef[1 + ng + (i - 1 - kMaxLin)];
    }
    for (int64_t r0 = static_cast<int64_t>(blockIdx.x) * kRowThreads; r0 < n;
         r0 += static_cast<int64_t>(gridDim.x) * kRowThreads) {
        __syncthreads();
        stage_rows(tile, genes, n, ldg, ng, st, r0);
        __syncthreads();
        if (r0 + threadIdx.x < n) {
            double g[kMaxLin];
#pragma unroll
            for (int k = 0; k < kMaxLin; ++k) g[k] = (k < ng) ? static_cast<double>(tile[threadIdx.x * st + k]) : 0.0;
            double s = c0;
#pragma unroll
            for (int k = 0; k < kMaxLin; ++k) s = fma(lin[k], g[k], s);
#pragma unroll
            for (int i = 0; i < kQuadGenes; ++i) {
                double t = 0.0;
#pragma unroll
                for (int j = 0; j <= i; ++j) t = fma(q[tri(i) + j], g[j], t);
                s = fma(t, g[i], s);
            }
            score[r0 + threadIdx.x] = s;
        }
    }
}

template <int P>
__global__ void __launch_bounds__(kRowThreads) sg_grad_genes_kernel(const float *__restrict__ coef, int ng,
                                                                    const float *__restrict__ genes, int64_t n,
                                                                    int ldg, const float *__restrict__ gout,
                                                                    float *__restrict__ dgenes) {
    __shared__ CoefF c;
    extern __shared__ float tile[];
    const int st = stride_for(ng);
    load_coef<P>(c, coef, ng);
    for (int64_t r0 = static_cast<int64_t>(blockIdx.x) * kRowThreads; r0 < n;
         r0 += static_cast<int64_t>(gridDim.x) * kRowThreads) {
        __syncthreads();
        stage_rows(tile, genes, n, ldg, ng, st, r0);
        __syncthreads();
        const int64_t r = r0 + threadIdx.x;
        float d[kMaxLin];
        if (r < n) {
            float g[kMaxLin];
            read_row<P>(g, tile, st, ng);
            grad_f32(c, g, d);
            const float go = gout[r];
#pragma unroll
            for (int k = 0; k < kMaxLin; ++k) d[k] = (k < ng) ? __fmul_rn(go, d[k]) : 0.0f;
        }
        __syncthreads();
        // write back through the tile so that the global stores are coalesced
        if (r < n) {
#pragma unroll
            for (int k = 0; k < kMaxLin; ++k)
                if (k < ng) tile[threadIdx.x * st + k] = d[k];
        }
        __syncthreads();
        const int64_t rows = (n - r0 < kRowThreads) ? (n - r0) : kRowThreads;
        const int total = static_cast<int>(rows) * ldg;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int rr = idx / ldg, k = idx - rr * ldg;
            dgenes[r0 * ldg + idx] = (k < ng) ? tile[rr * st + k] : 0.0f;
        }
    }
}

// Feature f as a product x[a]·x[b] over x = [g_0 .. g_{ng-1}, 1].
__device__ __forceinline__ void feature_pair(int f, int ng, int &a, int &b) {
    if (f == 0) {
        a = ng;
        b = ng;
    } else if (f <= ng) {
        a = f - 1;
        b = ng;
    } else {
        int q = f - 1 - ng, i = 0;
        while (tri(i + 1) <= q) ++i;
        a = i;
        b = q - tri(i);
    }
}

// Per-block partial sums of Σ_r gout_r Φ_f(g_r), FP64, thread f per feature.
template <typename TG>
__global__ void __launch_bounds__(kRowThreads) sg_grad_coef_kernel(int ng, int nf, const float *__restrict__ genes,
                                                                   int64_t n, int ldg, const TG *__restrict__ gout,
                                                                   double *__restrict__ part) {
    extern __shared__ float tile[];
    __shared__ double go_s[kRowThreads];
    const int st = stride_for(ng);
    int a = 0, b = 0;
    if (threadIdx.x < nf) feature_pair(threadIdx.x, ng, a, b);
    double acc = 0.0;
    for (int64_t r0 = static_cast<int64_t>(blockIdx.x) * kRowThreads; r0 < n;
         r0 += static_cast<int64_t>(gridDim.x) * kRowThreads) {
        __syncthreads();
        stage_rows(tile, genes, n, ldg, ng, st, r0);
        const int64_t rows = (n - r0 < kRowThreads) ? (n - r0) : kRowThreads;
        if (threadIdx.x < rows) {
            tile[threadIdx.x * st + ng] = 1.0f;
            go_s[threadIdx.x] = static_cast<double>(gout[r0 + threadIdx.x]);
        }
        __syncthreads();
        if (threadIdx.x < nf) {
            for (int r = 0; r < rows; ++r) {
                const double phi = static_cast<double>(tile[r * st + a]) * static_cast<double>(tile[r * st + b]);
                acc = fma(go_s[r], phi, acc);
            }
        }
    }
    if (threadIdx.x < nf) part[static_cast<int64_t>(blockIdx.x) * kMaxFeat + threadIdx.x] = acc;
}

__global__ void sg_sum_parts_kernel(const double *__restrict__ part, int nparts, int stride, int nf,
                                    double *__restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += part[static_cast<int64_t>(p) * stride + f];
    out[f] = s;
}

// Normal equations: thread t owns the 4×4 block (bi, bj), bj <= bi, of ΦᵀΦ;
// threads t < nf also accumulate (Φᵀy)_t. Φ for kGramRows rows is staged in
// shared memory in FP64 (exact: a product of two f32 genes).
__global__ void __launch_bounds__(1024) sg_gram_kernel(int ng, int nf, const float *__restrict__ genes, int64_t n,
                                                       int ldg, const double *__restrict__ fit,
                                                       double *__restrict__ part_g, double *__restrict__ part_r) {
    extern __shared__ double phi[];  // [kGramRows][kGramFeatPad]
    __shared__ float gs[kGramRows][kMaxLin + 1];
    __shared__ double ys[kGramRows];
    const int nb = (nf + kGramBlk - 1) / kGramBlk;
    const int npairs = nb * (nb + 1) / 2;
    const int t = threadIdx.x;
    int bi = 0;
    while (tri(bi + 1) <= t) ++bi;
    const int bj = t - tri(bi);
    const bool owner = t < npairs;
    int fa = 0, fb = 0;
    if (t < nf) feature_pair(t, ng, fa, fb);
    double acc[kGramBlk][kGramBlk] = {};
    double racc = 0.0;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = static_cast<int64_t>(blockIdx.x) * chunk;
    const int64_t hi = (lo + chunk < n) ? lo + chunk : n;
    for (int64_t r0 = lo; r0 < hi; r0 += kGramRows) {
        const int rows = static_cast<int>((hi - r0 < kGramRows) ? hi - r0 : kGramRows);
        __syncthreads();
        for (int idx = t; idx < rows * ng; idx += blockDim.x) {
            const int r = idx / ng, k = idx - r * ng;
            gs[r][k] = genes[(r0 + r) * static_cast<int64_t>(ldg) + k];
        }
        if (t < rows) {
            gs[t][ng] = 1.0f;
            ys[t] = fit ? fit[r0 + t] : 0.0;
        }
        __syncthreads();
        for (int idx = t; idx < kGramRows * kGramFeatPad; idx += blockDim.x) {
            const int r = idx / kGramFeatPad, f = idx - r * kGramFeatPad;
            double v = 0.0;
            if (r < rows && f < nf) {
                int a, b;
                feature_pair(f, ng, a, b);
                v = static_cast<double>(gs[r][a]) * static_cast<double>(gs[r][b]);
            }
            phi[idx] = v;
        }
        __syncthreads();
        if (owner) {
            for (int r = 0; r < rows; ++r) {
                const double *pr = phi + r * kGramFeatPad;
                double xa[kGramBlk], xb[kGramBlk];
#pragma unroll
                for (int u = 0; u < kGramBlk; ++u) {
                    xa[u] = pr[bi * kGramBlk + u];
                    xb[u] = pr[bj * kGramBlk + u];
                }
#pragma unroll
                for (int u = 0; u < kGramBlk; ++u)
#pragma unroll
                    for (int v = 0; v < kGramBlk; ++v) acc[u][v] = fma(xa[u], xb[v], acc[u][v]);
            }
        }
        if (t < nf && fit) {
            for (int r = 0; r < rows; ++r) racc = fma(ys[r], phi[r * kGramFeatPad + t], racc);
        }
    }
    if (owner) {
        double *dst = part_g + (static_cast<int64_t>(blockIdx.x) * kGramPairs + t) * (kGramBlk * kGramBlk);
#pragma unroll
        for (int u = 0; u < kGramBlk; ++u)
#pragma unroll
            for (int v = 0; v < kGramBlk; ++v) dst[u * kGramBlk + v] = acc[u][v];
    }
    if (t < nf) part_r[static_cast<int64_t>(blockIdx.x) * kMaxFeat + t] = racc;
}

__global__ void sg_gram_sum_kernel(const double *__restrict__ part_g, int nparts, int nf, double *__restrict__ gram) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // (pair, u, v)
    const int nb = (nf + kGramBlk - 1) / kGramBlk;
    const int npairs = nb * (nb + 1) / 2;
    if (e >= npairs * kGramBlk * kGramBlk) return;
    const int t = e / (kGramBlk * kGramBlk), uv = e - t * (kGramBlk * kGramBlk);
    const int u = uv / kGramBlk, v = uv - u * kGramBlk;
    int bi = 0;
    while (tri(bi + 1) <= t) ++bi;
    const int bj = t - tri(bi);
    const int a = bi * kGramBlk + u, b = bj * kGramBlk + v;
    if (a >= nf || b >= nf) return;
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += part_g[(static_cast<int64_t>(p) * kGramPairs + t) * (kGramBlk * kGramBlk) + uv];
    gram[static_cast<int64_t>(a) * nf + b] = s;
    gram[static_cast<int64_t>(b) * nf + a] = s;
}

// (G + αI) w = rhs + α·prior by Cholesky, FP64, packed lower triangle in
// shared memory, one CTA of 32×32 threads.
__global__ void __launch_bounds__(kSolveThreads) sg_ridge_solve_kernel(int n, const double *__restrict__ gram,
                                                                       const double *__restrict__ rhs, double alpha,
                                                                       const double *__restrict__ prior,
                                                                       double *__restrict__ w, int *status) {
    extern __shared__ double L[];  // tri(n) entries, then y[n]
    double *y = L + tri(n);
    __shared__ int bad;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    if (tid == 0) bad = 0;
    for (int i = ty; i < n; i += 32)
        for (int j = tx; j <= i; j += 32) L[tri(i) + j] = gram[static_cast<int64_t>(i) * n + j] + (i == j ? alpha : 0.0);
    for (int i = tid; i < n; i += kSolveThreads) y[i] = rhs[i] + (prior ? alpha * prior[i] : 0.0);
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (tid == 0) {
            const double d = L[tri(k) + k];
            if (!(d > 0.0) && bad == 0) bad = k + 1;
            L[tri(k) + k] = sqrt(d);
        }
        __syncthreads();
        const double p = L[tri(k) + k];
        for (int i = k + 1 + tid; i < n; i += kSolveThreads) L[tri(i) + k] /= p;
        __syncthreads();
        for (int i = k + 1 + ty; i < n; i += 32) {
            const double lik = L[tri(i) + k];
            for (int j = k + 1 + tx; j <= i; j += 32) L[tri(i) + j] = fma(-lik, L[tri(j) + k], L[tri(i) + j]);
        }
        __syncthreads();
    }
    for (int j = 0; j < n; ++j) {  // L z = y
        if (tid == 0) y[j] /= L[tri(j) + j];
        __syncthreads();
        const double yj = y[j];
        for (int i = j + 1 + tid; i < n; i += kSolveThreads) y[i] = fma(-L[tri(i) + j], yj, y[i]);
        __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {  // Lᵀ w = z
        if (tid == 0) y[j] /= L[tri(j) + j];
        __syncthreads();
        const double yj = y[j];
        for (int i = tid; i < j; i += kSolveThreads) y[i] = fma(-L[tri(j) + i], yj, y[i]);
        __syncthreads();
    }
    for (int i = tid; i < n; i += kSolveThreads) w[i] = y[i];
    if (tid == 0) *status = bad;
}

__global__ void __launch_bounds__(kRowThreads) sg_ascend_kernel(const float *__restrict__ coef, int ng,
                                                                float *__restrict__ genes, int64_t n, int ldg,
                                                                float eta, int steps, float *__restrict__ score) {
    __shared__ CoefF c;
    extern __shared__ float tile[];
    const int st = stride_for(ng);
    load_coef<CSX_SG_FP32>(c, coef, ng);
    for (int64_t r0 = static_cast<int64_t>(blockIdx.x) * kRowThreads; r0 < n;
         r0 += static_cast<int64_t>(gridDim.x) * kRowThreads) {
        __syncthreads();
        stage_rows(tile, genes, n, ldg, ng, st, r0);
        __syncthreads();
        const int64_t r = r0 + threadIdx.x;
        if (r < n) {
            float g[kMaxLin], d[kMaxLin];
            read_row<CSX_SG_FP32>(g, tile, st, ng);
            for (int s = 0; s < steps; ++s) {
                grad_f32(c, g, d);
#pragma unroll
                for (int k = 0; k < kMaxLin; ++k)
                    if (k < ng) g[k] = fmaxf(fminf(__fmaf_rn(eta, d[k], g[k]), 1.0f), 0.0f);
            }
            if (score) score[r] = score_f32(c, g);
#pragma unroll
            for (int k = 0; k < kMaxLin; ++k)
                if (k < ng) tile[threadIdx.x * st + k] = g[k];
        }
        __syncthreads();
        const int64_t rows = (n - r0 < kRowThreads) ? (n - r0) : kRowThreads;
        const int total = static_cast<int>(rows) * ng;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int rr = idx / ng, k = idx - rr * ng;
            genes[(r0 + rr) * static_cast<int64_t>(ldg) + k] = tile[rr * st + k];
        }
    }
}

#define SG_CUDA(call)                                                                       \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            std::fprintf(stderr, "csx: %s failed: %s\n", #call, cudaGetErrorString(e_));   \
            return e_ == cudaErrorMemoryAllocation ? CSX_ERR_OOM : CSX_ERR_CUDA;             \
        }                                                                                   \
    } while (0)

int check_layout(int nf, int ldg, int64_t n, int &ng) {
    if (nf < kMinFeat || nf > kMaxFeat || n < 0) return CSX_ERR_BAD_ARGS;
    ng = nf - 1 - kNQuad;
    if (ldg < ng) return CSX_ERR_BAD_ARGS;
    return CSX_OK;
}

int row_grid(int64_t n) {
    const int64_t tiles = (n + kRowThreads - 1) / kRowThreads;
    const int64_t cap = 152 * 8;
    return static_cast<int>(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
}

size_t tile_bytes(int ng) { return static_cast<size_t>(kRowThreads) * stride_for(ng) * sizeof(float); }

constexpr size_t kPartCoefBytes = static_cast<size_t>(kPartBlocks) * kMaxFeat * sizeof(double);
constexpr size_t kPartGramBytes = static_cast<size_t>(kPartBlocks) * kGramPairs * kGramBlk * kGramBlk * sizeof(double);
constexpr size_t kGramSmem = static_cast<size_t>(kGramRows) * kGramFeatPad * sizeof(double);
constexpr size_t kSolveSmem = (static_cast<size_t>(tri(kMaxFeat)) + kMaxFeat) * sizeof(double);

int enable_solve_smem() {  // on the current device, every call (cheap)
    SG_CUDA(cudaFuncSetAttribute(sg_ridge_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kSolveSmem)));
    return CSX_OK;
}

template <typename TG>
int coef_grad(int ng, int nf, const float *genes, int64_t n, int ldg, const TG *gout, double *dcoef, void *work,
              cudaStream_t s) {
    if (!dcoef) return CSX_OK;
    if (!work) return CSX_ERR_BAD_ARGS;
    auto *part = static_cast<double *>(work);
    const int grid = static_cast<int>(n > 0 ? ((n + kRowThreads - 1) / kRowThreads < kPartBlocks
                                                   ? (n + kRowThreads - 1) / kRowThreads
                                                   : kPartBlocks)
                                            : 1);
    sg_grad_coef_kernel<TG><<<grid, kRowThreads, tile_bytes(ng), s>>>(ng, nf, genes, n, ldg, gout, part);
    SG_CUDA(cudaGetLastError());
    sg_sum_parts_kernel<<<1, 256, 0, s>>>(part, grid, kMaxFeat, nf, dcoef);
    SG_CUDA(cudaGetLastError());
    return CSX_OK;
}

}  // namespace

extern "C" {

uint64_t csx_sg_workspace_bytes(int nf) {
    (void)nf;
    return static_cast<uint64_t>(kPartGramBytes + kPartCoefBytes);
}

int csx_sg_forward(const float *d_coef, int nf, const float *d_genes, int64_t n, int ldg, int precision,
                   float *d_score, void *stream) {
    int ng = 0;
    if (int rc = check_layout(nf, ldg, n, ng)) return rc;
    if (n == 0) return CSX_OK;
    if (!d_coef || !d_genes || !d_score) return CSX_ERR_BAD_ARGS;
    auto s = static_cast<cudaStream_t>(stream);
    const int grid = row_grid(n);
    if (precision == CSX_SG_FP32) {
        sg_forward_kernel<CSX_SG_FP32><<<grid, kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg, d_score);
    } else if (precision == CSX_SG_BF16) {
        sg_forward_kernel<CSX_SG_BF16><<<grid, kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg, d_score);
    } else {
        return CSX_ERR_BAD_ARGS;
    }
    SG_CUDA(cudaGetLastError());
    return CSX_OK;
}

int csx_sg_forward_f64(const double *d_coef, int nf, const float *d_genes, int64_t n, int ldg, double *d_score,
                       void *stream) {
    int ng = 0;
    if (int rc = check_layout(nf, ldg, n, ng)) return rc;
    if (n == 0) return CSX_OK;
    if (!d_coef || !d_genes || !d_score) return CSX_ERR_BAD_ARGS;
    auto s = static_cast<cudaStream_t>(stream);
    sg_forward_f64_kernel<<<row_grid(n), kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg, d_score);
    SG_CUDA(cudaGetLastError());
    return CSX_OK;
}

int csx_sg_backward(const float *d_coef, int nf, const float *d_genes, int64_t n, int ldg, int precision,
                    const float *d_gout, float *d_dgenes, double *d_dcoef, void *d_work, void *stream) {
    int ng = 0;
    if (int rc = check_layout(nf, ldg, n, ng)) return rc;
    if (precision != CSX_SG_FP32 && precision != CSX_SG_BF16) return CSX_ERR_BAD_ARGS;
    if (n > 0 && (!d_genes || !d_gout || (d_dgenes && !d_coef))) return CSX_ERR_BAD_ARGS;
    auto s = static_cast<cudaStream_t>(stream);
    if (d_dgenes && n > 0) {
        const int grid = row_grid(n);
        if (precision == CSX_SG_FP32)
            sg_grad_genes_kernel<CSX_SG_FP32><<<grid, kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                       d_gout, d_dgenes);
        else
            sg_grad_genes_kernel<CSX_SG_BF16><<<grid, kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                       d_gout, d_dgenes);
        SG_CUDA(cudaGetLastError());
    }
    return coef_grad<float>(ng, nf, d_genes, n, ldg, d_gout, d_dcoef, d_work, s);
}

int csx_sg_backward_coef_f64(int nf, const float *d_genes, int64_t n, int ldg, const double *d_gout, double *d_dcoef,
                             void *d_work, void *stream) {
    int ng = 0;
    if (int rc = check_layout(nf, ldg, n, ng)) return rc;
    if (n > 0 && (!d_genes || !d_gout)) return CSX_ERR_BAD_ARGS;
    return coef_grad<double>(ng, nf, d_genes, n, ldg, d_gout, d_dcoef, d_work, static_cast<cudaStream_t>(stream));
}

int csx_sg_normal_equations(int nf, const float *d_genes, int64_t n, int ldg, const double *d_fit, double *d_gram,
                            double *d_rhs, void *d_work, void *stream) {
    int ng = 0;
    if (int rc = check_layout(nf, ldg, n, ng)) return rc;
    if (!d_gram || !d_work || (n > 0 && !d_genes) || (d_fit && !d_rhs)) return CSX_ERR_BAD_ARGS;
    auto s = static_cast<cudaStream_t>(stream);
    auto *part_g = static_cast<double *>(d_work);
    auto *part_r = reinterpret_cast<double *>(static_cast<char *>(d_work) + kPartGramBytes);
    const int nb = (nf + kGramBlk - 1) / kGramBlk;
    const int npairs = nb * (nb + 1) / 2;
    const int threads = ((npairs > nf ? npairs : nf) + 31) / 32 * 32;
    const int64_t want = (n + kGramRows - 1) / kGramRows;
    const int grid = static_cast<int>(want < kPartBlocks ? (want > 0 ? want : 1) : kPartBlocks);
    sg_gram_kernel<<<grid, threads, kGramSmem, s>>>(ng, nf, d_genes, n, ldg, d_fit, part_g, part_r);
    SG_CUDA(cudaGetLastError());
    const int ne = npairs * kGramBlk * kGramBlk;
    sg_gram_sum_kernel<<<(ne + 255) / 256, 256, 0, s>>>(part_g, grid, nf, d_gram);
    SG_CUDA(cudaGetLastError());
    if (d_fit) {
        sg_sum_parts_kernel<<<1, 256, 0, s>>>(part_r, grid, kMaxFeat, nf, d_rhs);
        SG_CUDA(cudaGetLastError());
    }
    return CSX_OK;
}

int csx_sg_ridge_solve(int nf, const double *d_gram, const double *d_rhs, double alpha, const double *d_prior,
                       double *d_w, int *d_status, void *stream) {
    if (nf < 1 || nf > kMaxFeat || !d_gram || !d_rhs || !d_w || !d_status || !(alpha >= 0.0)) return CSX_ERR_BAD_ARGS;
    if (int rc = enable_solve_smem()) return rc;
    const size_t smem = (static_cast<size_t>(tri(nf)) + nf) * sizeof(double);
    sg_ridge_solve_kernel<<<1, kSolveThreads, smem, static_cast<cudaStream_t>(stream)>>>(nf, d_gram, d_rhs, alpha,
                                                                                        d_prior, d_w, d_status);
    SG_CUDA(cudaGetLastError());
    return CSX_OK;
}

int csx_sg_ascend(const float *d_coef, int nf, float *d_genes, int64_t n, int ldg, float eta, int steps,
                  float *d_score, void *stream) {
    int ng = 0;
    if (int rc = check_layout(nf, ldg, n, ng)) return rc;
    if (steps < 0) return CSX_ERR_BAD_ARGS;
    if (n == 0) return CSX_OK;
    if (!d_coef || !d_genes) return CSX_ERR_BAD_ARGS;
    auto s = static_cast<cudaStream_t>(stream);
    sg_ascend_kernel<<<row_grid(n), kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg, eta, steps,
                                                                     d_score);
    SG_CUDA(cudaGetLastError());
    return CSX_OK;
}

}  // extern "C"
