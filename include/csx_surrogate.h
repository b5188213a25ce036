/*
 * csx_surrogate.h — the quadratic surrogate as a differentiable function on
 * the GPU: batched forward, hand-written backward (d score / d genes and
 * d loss / d coefficients), the ridge refit's normal equations and an FP64
 * Cholesky solve, and a gradient-guided mutation step.
 *
 * These replace brain/evolve.py:211-268 (features, refit_surrogate: numpy
 * FP64 `solve((XᵀX + αI), Xᵀy + αw₀)`) and give the screen's surrogate
 * (src/screen.zig:97-112) a gradient. Nothing in the reference computes a
 * gradient; the mutation step is new.
 *
 * Coefficient layout (compact, as brain/evolve.py:211-220 and
 * src/screen.zig:36-95 write it): nf = 1 + ng + 136 floats,
 *   [0]            constant
 *   [1 .. ng]      linear terms of genes 0..ng-1 (16 <= ng <= 29)
 *   [1+ng .. nf)   quadratic terms g_i·g_j over genes 0..15, (i, j <= i),
 *                  i outer, j inner.
 * nf = 153 is the v1 layout (16 genes), 166 the v6 layout (29 genes).
 * nf = 465 is the full surface of csx_screen.h (CSX_FULL_NF): 29 linear terms
 * and the quadratic terms over all 29 genes, (i, j <= i), i outer; its FP32
 * forward evaluates csx_score_full's FMA order.
 *
 * Genes: n rows of ldg floats (ldg >= ng); only the first ng are read.
 * Every pointer named d_* is device memory; `stream` is a cudaStream_t
 * (NULL = the legacy default stream). All calls are asynchronous on that
 * stream and return CSX_OK once enqueued, or an argument / CUDA status from
 * csx_screen.h.
 */
#ifndef CSX_SURROGATE_H
#define CSX_SURROGATE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CSX_SG_FP32 0 /* FP32 features and FMA accumulation */
#define CSX_SG_BF16 1 /* genes and coefficients rounded to bf16, FP32 accumulation */
#define CSX_SG_FP64 2 /* FP64 throughout */

/* Bytes of device workspace the d_dcoef and normal-equation reductions need
   for nf coefficients (deterministic two-stage reductions). */
uint64_t csx_sg_workspace_bytes(int nf);

/* score[r] = Φ(g_r)·coef in the given precision (FP64 precision writes
   float scores rounded from the FP64 sum). */
int csx_sg_forward(const float *d_coef, int nf, const float *d_genes, int64_t n, int ldg, int precision,
                   float *d_score, void *stream);

/* FP64 forward: score[r] = Φ(g_r)·coef with coef in FP64 (the ridge loss
   residual). */
int csx_sg_forward_f64(const double *d_coef, int nf, const float *d_genes, int64_t n, int ldg,
                       double *d_score, void *stream);

/* Backward of forward():
     d_dgenes[r*ldg + k] = gout[r] · ∂score/∂g_k   (k < ng; k >= ng written 0),
     d_dcoef[f]          = Σ_r gout[r] · Φ_f(g_r)  (FP64, fixed summation order).
   Either output may be NULL. The FP32/BF16 gene gradient is evaluated in the
   forward's precision; d_dcoef always accumulates in FP64. d_work holds
   csx_sg_workspace_bytes(nf). */
int csx_sg_backward(const float *d_coef, int nf, const float *d_genes, int64_t n, int ldg, int precision,
                    const float *d_gout, float *d_dgenes, double *d_dcoef, void *d_work, void *stream);

/* Same with an FP64 upstream gradient (the ridge residual). */
int csx_sg_backward_coef_f64(int nf, const float *d_genes, int64_t n, int ldg, const double *d_gout,
                             double *d_dcoef, void *d_work, void *stream);

/* Normal equations of the ridge refit, FP64: d_gram (nf×nf, row-major, full
   symmetric) = ΦᵀΦ, d_rhs (nf) = Φᵀy. d_fit may be NULL (rhs not written). */
int csx_sg_normal_equations(int nf, const float *d_genes, int64_t n, int ldg, const double *d_fit,
                            double *d_gram, double *d_rhs, void *d_work, void *stream);

/* Ridge solve in FP64 by Cholesky on one CTA: w = (G + αI)⁻¹ (rhs + α·prior).
   d_prior may be NULL (zero prior). d_status (one int) receives 0, or k+1
   when the k-th pivot is not positive. nf <= 166, or 465 (the factor then
   lives in a scratch allocated and freed on `stream`). */
int csx_sg_ridge_solve(int nf, const double *d_gram, const double *d_rhs, double alpha, const double *d_prior,
                       double *d_w, int *d_status, void *stream);

/* Gradient-guided mutation: `steps` projected gradient-ascent steps
   g <- clamp01(g + eta·∇score(g)) on the first ng genes of every row (FP32),
   in place; d_score (may be NULL) receives the final FP32 scores. */
int csx_sg_ascend(const float *d_coef, int nf, float *d_genes, int64_t n, int ldg, float eta, int steps,
                  float *d_score, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CSX_SURROGATE_H */
