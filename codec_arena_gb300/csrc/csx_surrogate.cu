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

constexpr int kQuadGenes = 16;                             // the reference layouts' quadratic block
constexpr int kNQuad = kQuadGenes * (kQuadGenes + 1) / 2;  // 136
constexpr int kMaxLin = 29;
constexpr int kMinFeat = 1 + kQuadGenes + kNQuad;  // 153
constexpr int kMaxFeat = 1 + kMaxLin + kNQuad;     // 166
// The full surface (csx_screen.h): the quadratic block over all 29 genes.
constexpr int kNQuadFull = kMaxLin * (kMaxLin + 1) / 2;  // 435
constexpr int kFullFeat = 1 + kMaxLin + kNQuadFull;      // 465
constexpr int kFeatCap = kFullFeat;                      // stride of per-feature partial sums
constexpr int kRowThreads = 256;                   // rows per tile in the row kernels
constexpr int kPartBlocks = 152;                   // fixed: the reductions' summation order never changes
constexpr int kPartBlocksFull = 64;                // the same for the full layout's normal equations
constexpr int kGramRows = 32;                      // rows per Φ tile in the normal equations
constexpr int kGramBlk = 4;                        // each thread owns a 4×4 block of ΦᵀΦ
constexpr int kGramThreads = 1024;                 // 4×4 blocks per CTA (CTAs along y split the blocks)
constexpr int kSolveThreads = 1024;

__host__ __device__ constexpr int tri(int i) { return i * (i + 1) / 2; }
__host__ __device__ constexpr int gram_nb(int nf) { return (nf + kGramBlk - 1) / kGramBlk; }
__host__ __device__ constexpr int gram_pairs(int nf) { return tri(gram_nb(nf)); }
constexpr int kGramFeatPadFull = gram_nb(kFullFeat) * kGramBlk;  // 468

// Coefficients as the row kernels read them: linear terms padded with zeros to
// 29, quadratic terms packed (i, j <= i) over the first QG genes (16: the
// reference's layouts; 29: the full surface).
template <int QG>
struct CoefT {
    float c0;
    float lin[kMaxLin];
    float q[QG * (QG + 1) / 2];
};

template <int P>
__device__ __forceinline__ float in_prec(float x) {
    if constexpr (P == CSX_SG_BF16) return __bfloat162float(__float2bfloat16_rn(x));
    return x;
}

template <int P, int QG>
__device__ void load_coef(CoefT<QG> &s, const float *coef, int ng) {
    constexpr int nq = QG * (QG + 1) / 2;
    for (int i = threadIdx.x; i < 1 + kMaxLin + nq; i += blockDim.x) {
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

// FP32 score. The reference layouts: linear terms, then the quadratic rows.
// The full surface: csx_screen.h's defined FMA order (the screen's score).
template <int QG>
__device__ __forceinline__ float score_f32(const CoefT<QG> &c, const float (&g)[kMaxLin]) {
    if constexpr (QG == kMaxLin) {
        float r = c.c0;
#pragma unroll
        for (int k = 0; k < kMaxLin; ++k) {
            float t = c.lin[k];
#pragma unroll
            for (int l = 0; l <= k; ++l) t = __fmaf_rn(c.q[tri(k) + l], g[l], t);
            r = __fmaf_rn(g[k], t, r);
        }
        return r;
    } else {
        float s = c.c0;
#pragma unroll
        for (int k = 0; k < kMaxLin; ++k) s = __fmaf_rn(c.lin[k], g[k], s);
#pragma unroll
        for (int i = 0; i < QG; ++i) {
            float t = 0.0f;
#pragma unroll
            for (int j = 0; j <= i; ++j) t = __fmaf_rn(c.q[tri(i) + j], g[j], t);
            s = __fmaf_rn(t, g[i], s);
        }
        return s;
    }
}

// ∂score/∂g_k = lin_k + Σ_{j<=k} q_kj g_j + Σ_{i>=k} q_ik g_i (k < QG).
template <int QG>
__device__ __forceinline__ void grad_f32(const CoefT<QG> &c, const float (&g)[kMaxLin], float (&d)[kMaxLin]) {
#pragma unroll
    for (int k = 0; k < kMaxLin; ++k) d[k] = c.lin[k];
#pragma unroll
    for (int i = 0; i < QG; ++i) {
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            const float q = c.q[tri(i) + j];
            d[i] = __fmaf_rn(q, g[j], d[i]);
            d[j] = __fmaf_rn(q, g[i], d[j]);
        }
    }
}

__host__ __device__ inline int stride_for(int ng) { return ((ng + 1) & 1) ? ng + 1 : ng + 2; }  // odd, >= ng + 1

template <int P, int QG>
__global__ void __launch_bounds__(kRowThreads) sg_forward_kernel(const float *__restrict__ coef, int ng,
                                                                 const float *__restrict__ genes, int64_t n,
                                                                 int ldg, float *__restrict__ score) {
    __shared__ CoefT<QG> c;
    extern __shared__ float tile[];
    const int st = stride_for(ng);
    load_coef<P, QG>(c, coef, ng);
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

template <int QG>
__global__ void __launch_bounds__(kRowThreads) sg_forward_f64_kernel(const double *__restrict__ coef, int ng,
                                                                     const float *__restrict__ genes, int64_t n,
                                                                     int ldg, double *__restrict__ score) {
    constexpr int nq = QG * (QG + 1) / 2;
    __shared__ double lin[kMaxLin], q[nq], c0;
    extern __shared__ float tile[];
    const int st = stride_for(ng);
    for (int i = threadIdx.x; i < 1 + kMaxLin + nq; i += blockDim.x) {
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
            for (int i = 0; i < QG; ++i) {
                double t = 0.0;
#pragma unroll
                for (int j = 0; j <= i; ++j) t = fma(q[tri(i) + j], g[j], t);
                s = fma(t, g[i], s);
            }
            score[r0 + threadIdx.x] = s;
        }
    }
}

template <int P, int QG>
__global__ void __launch_bounds__(kRowThreads) sg_grad_genes_kernel(const float *__restrict__ coef, int ng,
                                                                    const float *__restrict__ genes, int64_t n,
                                                                    int ldg, const float *__restrict__ gout,
                                                                    float *__restrict__ dgenes) {
    __shared__ CoefT<QG> c;
    extern __shared__ float tile[];
    const int st = stride_for(ng);
    load_coef<P, QG>(c, coef, ng);
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
    constexpr int kPer = (kFeatCap + kRowThreads - 1) / kRowThreads;  // features per thread (2)
    extern __shared__ float tile[];
    __shared__ double go_s[kRowThreads];
    const int st = stride_for(ng);
    int a[kPer], b[kPer];
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        a[m] = b[m] = 0;
        const int f = threadIdx.x + m * kRowThreads;
        if (f < nf) feature_pair(f, ng, a[m], b[m]);
    }
    double acc[kPer] = {};
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
#pragma unroll
        for (int m = 0; m < kPer; ++m) {
            if (threadIdx.x + m * kRowThreads < nf) {
                for (int r = 0; r < rows; ++r) {
                    const double phi =
                        static_cast<double>(tile[r * st + a[m]]) * static_cast<double>(tile[r * st + b[m]]);
                    acc[m] = fma(go_s[r], phi, acc[m]);
                }
            }
        }
    }
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        const int f = threadIdx.x + m * kRowThreads;
        if (f < nf) part[static_cast<int64_t>(blockIdx.x) * kFeatCap + f] = acc[m];
    }
}

__global__ void sg_sum_parts_kernel(const double *__restrict__ part, int nparts, int stride, int nf,
                                    double *__restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += part[static_cast<int64_t>(p) * stride + f];
    out[f] = s;
}

// Normal equations: thread t of CTA column y owns the 4×4 block number
// y·1024 + t, (bi, bj) with bj <= bi, of ΦᵀΦ; CTA row x accumulates rows of
// its chunk. Column 0's threads t < nf also accumulate (Φᵀy)_t. Φ for
// kGramRows rows is staged in shared memory in FP64 (exact: a product of two
// f32 genes), featpad = 4·ceil(nf/4) features per row.
__global__ void __launch_bounds__(kGramThreads) sg_gram_kernel(int ng, int nf, const float *__restrict__ genes,
                                                               int64_t n, int ldg, const double *__restrict__ fit,
                                                               double *__restrict__ part_g,
                                                               double *__restrict__ part_r) {
    extern __shared__ double phi[];  // [kGramRows][featpad]
    __shared__ float gs[kGramRows][kMaxLin + 1];
    __shared__ double ys[kGramRows];
    __shared__ unsigned char fa[kGramFeatPadFull], fb[kGramFeatPadFull];  // feature f = x[fa]·x[fb]
    const int nb = gram_nb(nf), featpad = nb * kGramBlk;
    const int npairs = tri(nb);
    const int t = threadIdx.x;
    for (int f = t; f < nf; f += blockDim.x) {
        int a, b;
        feature_pair(f, ng, a, b);
        fa[f] = static_cast<unsigned char>(a);
        fb[f] = static_cast<unsigned char>(b);
    }
    const int pt = blockIdx.y * kGramThreads + t;  // this thread's block number
    int bi = 0;
    while (tri(bi + 1) <= pt) ++bi;
    const int bj = pt - tri(bi);
    const bool owner = pt < npairs;
    const bool rhs_here = blockIdx.y == 0 && t < nf && fit;
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
        for (int idx = t; idx < kGramRows * featpad; idx += blockDim.x) {
            const int r = idx / featpad, f = idx - r * featpad;
            double v = 0.0;
            if (r < rows && f < nf) v = static_cast<double>(gs[r][fa[f]]) * static_cast<double>(gs[r][fb[f]]);
            phi[idx] = v;
        }
        __syncthreads();
        if (owner) {
            for (int r = 0; r < rows; ++r) {
                const double *pr = phi + r * featpad;
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
        if (rhs_here) {
            for (int r = 0; r < rows; ++r) racc = fma(ys[r], phi[r * featpad + t], racc);
        }
    }
    if (owner) {
        double *dst = part_g + (static_cast<int64_t>(blockIdx.x) * npairs + pt) * (kGramBlk * kGramBlk);
#pragma unroll
        for (int u = 0; u < kGramBlk; ++u)
#pragma unroll
            for (int v = 0; v < kGramBlk; ++v) dst[u * kGramBlk + v] = acc[u][v];
    }
    if (rhs_here) part_r[static_cast<int64_t>(blockIdx.x) * kFeatCap + t] = racc;
}

__global__ void sg_gram_sum_kernel(const double *__restrict__ part_g, int nparts, int nf, double *__restrict__ gram) {
    const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;  // (pair, u, v)
    const int npairs = gram_pairs(nf);
    if (e >= static_cast<int64_t>(npairs) * kGramBlk * kGramBlk) return;
    const int t = static_cast<int>(e / (kGramBlk * kGramBlk)), uv = static_cast<int>(e % (kGramBlk * kGramBlk));
    const int u = uv / kGramBlk, v = uv - u * kGramBlk;
    int bi = 0;
    while (tri(bi + 1) <= t) ++bi;
    const int bj = t - tri(bi);
    const int a = bi * kGramBlk + u, b = bj * kGramBlk + v;
    if (a >= nf || b >= nf) return;
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += part_g[(static_cast<int64_t>(p) * npairs + t) * (kGramBlk * kGramBlk) + uv];
    gram[static_cast<int64_t>(a) * nf + b] = s;
    gram[static_cast<int64_t>(b) * nf + a] = s;
}

// (G + αI) w = rhs + α·prior by Cholesky, FP64, packed lower triangle L
// (tri(n) entries, then y[n]) in shared memory up to 166 coefficients, in a
// global scratch for the full surface's 465; one CTA of 32×32 threads.
__device__ void ridge_solve_body(double *L, int n, const double *__restrict__ gram, const double *__restrict__ rhs,
                                 double alpha, const double *__restrict__ prior, double *__restrict__ w,
                                 int *status) {
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

__global__ void __launch_bounds__(kSolveThreads) sg_ridge_solve_kernel(int n, const double *__restrict__ gram,
                                                                       const double *__restrict__ rhs, double alpha,
                                                                       const double *__restrict__ prior,
                                                                       double *__restrict__ w, int *status) {
    extern __shared__ double L[];
    ridge_solve_body(L, n, gram, rhs, alpha, prior, w, status);
}

__global__ void __launch_bounds__(kSolveThreads) sg_ridge_solve_global_kernel(int n, const double *__restrict__ gram,
                                                                              const double *__restrict__ rhs,
                                                                              double alpha,
                                                                              const double *__restrict__ prior,
                                                                              double *__restrict__ w, int *status,
                                                                              double *scratch) {
    ridge_solve_body(scratch, n, gram, rhs, alpha, prior, w, status);
}

template <int QG>
__global__ void __launch_bounds__(kRowThreads) sg_ascend_kernel(const float *__restrict__ coef, int ng,
                                                                float *__restrict__ genes, int64_t n, int ldg,
                                                                float eta, int steps, float *__restrict__ score) {
    __shared__ CoefT<QG> c;
    extern __shared__ float tile[];
    const int st = stride_for(ng);
    load_coef<CSX_SG_FP32, QG>(c, coef, ng);
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
                // keep the coefficient loads inside the loop: hoisted, the full
                // surface's 435 quadratic terms would not fit in registers
                asm volatile("" ::: "memory");
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

// nf -> genes: the reference layouts (153..166: 16-gene quadratic block, ng
// genes linear) or the full surface (465: 29 genes, all quadratic).
int check_layout(int nf, int ldg, int64_t n, int &ng) {
    if (n < 0) return CSX_ERR_BAD_ARGS;
    if (nf == kFullFeat) {
        ng = kMaxLin;
    } else {
        if (nf < kMinFeat || nf > kMaxFeat) return CSX_ERR_BAD_ARGS;
        ng = nf - 1 - kNQuad;
    }
    if (ldg < ng) return CSX_ERR_BAD_ARGS;
    return CSX_OK;
}

bool is_full(int nf) { return nf == kFullFeat; }

int row_grid(int64_t n) {
    const int64_t tiles = (n + kRowThreads - 1) / kRowThreads;
    const int64_t cap = 152 * 8;
    return static_cast<int>(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
}

size_t tile_bytes(int ng) { return static_cast<size_t>(kRowThreads) * stride_for(ng) * sizeof(float); }

int gram_parts(int nf) { return is_full(nf) ? kPartBlocksFull : kPartBlocks; }
size_t part_gram_bytes(int nf) {
    return static_cast<size_t>(gram_parts(nf)) * gram_pairs(nf) * kGramBlk * kGramBlk * sizeof(double);
}
constexpr size_t kPartCoefBytes = static_cast<size_t>(kPartBlocks) * kFeatCap * sizeof(double);
size_t gram_smem(int nf) { return static_cast<size_t>(kGramRows) * gram_nb(nf) * kGramBlk * sizeof(double); }
constexpr size_t kSolveSmem = (static_cast<size_t>(tri(kMaxFeat)) + kMaxFeat) * sizeof(double);

int enable_smem() {  // on the current device, every call (cheap)
    SG_CUDA(cudaFuncSetAttribute(sg_ridge_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kSolveSmem)));
    SG_CUDA(cudaFuncSetAttribute(sg_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(gram_smem(kFullFeat))));
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
    sg_sum_parts_kernel<<<(nf + 255) / 256, 256, 0, s>>>(part, grid, kFeatCap, nf, dcoef);
    SG_CUDA(cudaGetLastError());
    return CSX_OK;
}

}  // namespace

extern "C" {

uint64_t csx_sg_workspace_bytes(int nf) {
    const size_t g = is_full(nf) ? part_gram_bytes(kFullFeat) : part_gram_bytes(kMaxFeat);
    return static_cast<uint64_t>(g + kPartCoefBytes);
}

int csx_sg_forward(const float *d_coef, int nf, const float *d_genes, int64_t n, int ldg, int precision,
                   float *d_score, void *stream) {
    int ng = 0;
    if (int rc = check_layout(nf, ldg, n, ng)) return rc;
    if (n == 0) return CSX_OK;
    if (!d_coef || !d_genes || !d_score) return CSX_ERR_BAD_ARGS;
    auto s = static_cast<cudaStream_t>(stream);
    const int grid = row_grid(n);
    const size_t tb = tile_bytes(ng);
    if (precision == CSX_SG_FP32) {
        if (is_full(nf))
            sg_forward_kernel<CSX_SG_FP32, kMaxLin><<<grid, kRowThreads, tb, s>>>(d_coef, ng, d_genes, n, ldg, d_score);
        else
            sg_forward_kernel<CSX_SG_FP32, kQuadGenes><<<grid, kRowThreads, tb, s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                    d_score);
    } else if (precision == CSX_SG_BF16) {
        if (is_full(nf))
            sg_forward_kernel<CSX_SG_BF16, kMaxLin><<<grid, kRowThreads, tb, s>>>(d_coef, ng, d_genes, n, ldg, d_score);
        else
            sg_forward_kernel<CSX_SG_BF16, kQuadGenes><<<grid, kRowThreads, tb, s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                    d_score);
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
    if (is_full(nf))
        sg_forward_f64_kernel<kMaxLin><<<row_grid(n), kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                      d_score);
    else
        sg_forward_f64_kernel<kQuadGenes><<<row_grid(n), kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n,
                                                                                         ldg, d_score);
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
        const size_t tb = tile_bytes(ng);
        const bool full = is_full(nf);
        if (precision == CSX_SG_FP32 && full)
            sg_grad_genes_kernel<CSX_SG_FP32, kMaxLin><<<grid, kRowThreads, tb, s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                    d_gout, d_dgenes);
        else if (precision == CSX_SG_FP32)
            sg_grad_genes_kernel<CSX_SG_FP32, kQuadGenes><<<grid, kRowThreads, tb, s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                       d_gout, d_dgenes);
        else if (full)
            sg_grad_genes_kernel<CSX_SG_BF16, kMaxLin><<<grid, kRowThreads, tb, s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                    d_gout, d_dgenes);
        else
            sg_grad_genes_kernel<CSX_SG_BF16, kQuadGenes><<<grid, kRowThreads, tb, s>>>(d_coef, ng, d_genes, n, ldg,
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
    if (int rc = enable_smem()) return rc;
    auto s = static_cast<cudaStream_t>(stream);
    auto *part_g = static_cast<double *>(d_work);
    auto *part_r = reinterpret_cast<double *>(static_cast<char *>(d_work) + part_gram_bytes(is_full(nf) ? kFullFeat
                                                                                                          : kMaxFeat));
    const int npairs = gram_pairs(nf);
    const int ycols = (npairs + kGramThreads - 1) / kGramThreads;
    const int threads = ycols > 1 ? kGramThreads : ((npairs > nf ? npairs : nf) + 31) / 32 * 32;
    const int64_t want = (n + kGramRows - 1) / kGramRows;
    const int cap = gram_parts(nf);
    const int grid = static_cast<int>(want < cap ? (want > 0 ? want : 1) : cap);
    sg_gram_kernel<<<dim3(grid, ycols), threads, gram_smem(nf), s>>>(ng, nf, d_genes, n, ldg, d_fit, part_g, part_r);
    SG_CUDA(cudaGetLastError());
    const int64_t ne = static_cast<int64_t>(npairs) * kGramBlk * kGramBlk;
    sg_gram_sum_kernel<<<static_cast<unsigned>((ne + 255) / 256), 256, 0, s>>>(part_g, grid, nf, d_gram);
    SG_CUDA(cudaGetLastError());
    if (d_fit) {
        sg_sum_parts_kernel<<<(nf + 255) / 256, 256, 0, s>>>(part_r, grid, kFeatCap, nf, d_rhs);
        SG_CUDA(cudaGetLastError());
    }
    return CSX_OK;
}

int csx_sg_ridge_solve(int nf, const double *d_gram, const double *d_rhs, double alpha, const double *d_prior,
                       double *d_w, int *d_status, void *stream) {
    if (nf < 1 || (nf > kMaxFeat && nf != kFullFeat) || !d_gram || !d_rhs || !d_w || !d_status || !(alpha >= 0.0))
        return CSX_ERR_BAD_ARGS;
    if (int rc = enable_smem()) return rc;
    auto s = static_cast<cudaStream_t>(stream);
    const size_t bytes = (static_cast<size_t>(tri(nf)) + nf) * sizeof(double);
    if (nf <= kMaxFeat) {
        sg_ridge_solve_kernel<<<1, kSolveThreads, bytes, s>>>(nf, d_gram, d_rhs, alpha, d_prior, d_w, d_status);
        SG_CUDA(cudaGetLastError());
        return CSX_OK;
    }
    // the full surface: the factor does not fit in shared memory
    void *scratch = nullptr;
    SG_CUDA(cudaMallocAsync(&scratch, bytes, s));
    sg_ridge_solve_global_kernel<<<1, kSolveThreads, 0, s>>>(nf, d_gram, d_rhs, alpha, d_prior, d_w, d_status,
                                                             static_cast<double *>(scratch));
    const cudaError_t e = cudaGetLastError();
    SG_CUDA(cudaFreeAsync(scratch, s));
    SG_CUDA(e);
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
    if (is_full(nf))
        sg_ascend_kernel<kMaxLin><<<row_grid(n), kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg, eta,
                                                                                 steps, d_score);
    else
        sg_ascend_kernel<kQuadGenes><<<row_grid(n), kRowThreads, tile_bytes(ng), s>>>(d_coef, ng, d_genes, n, ldg,
                                                                                    eta, steps, d_score);
    SG_CUDA(cudaGetLastError());
    return CSX_OK;
}

}  // extern "C"
