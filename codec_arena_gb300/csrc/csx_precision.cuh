// csx_precision.cuh — the precision form's model, its certified error bound,
// and tensor-core scoring of given genomes (csx_tc_score).
// Part of csx_screen.cu's translation unit (included there, in order); not a
// standalone header.
#pragma once

// ---- precision form: tensor-core scoring -------------------------------------------
namespace csx {

// The precision form of a model (FP64 on the host, then rounded): BF16 keeps
// x = g and L; FP16 uses x' = 2g - 1 in [-1, 1] and L/4, with the linear
// and constant parts of the substitution folded into the FP32 terms:
//   sum_{j<=i} L_ij g_i g_j = sum_i x'_i (L/4 x')_i + sum_i u_i x'_i + v,
//   u_i = (row sum + column sum of L at i) / 4, v = sum L / 4, x'_i = 2 g_i - 1.
int make_tc_model(const csx_model &m, bool fp16, TcModel *t) {
    double L[16][16] = {};
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) L[i][j] = m.w_quad[i * 16 + j];
    double c = 16.0 * static_cast<double>(m.w0);  // Model.score counts w0 once per legacy gene
    double lin[kNtot];
    for (int k = 0; k < kNtot; ++k) lin[k] = m.w_lin[k];
    double scale = 1.0;
    if (fp16) {
        double u[16] = {}, v = 0.0;
        for (int i = 0; i < 16; ++i)
            for (int j = 0; j <= i; ++j) {
                u[i] += L[i][j] / 4.0;
                u[j] += L[i][j] / 4.0;
                v += L[i][j] / 4.0;
            }
        for (int i = 0; i < 16; ++i) {
            lin[i] += 2.0 * u[i];
            c -= u[i];
        }
        c += v;
        scale = 0.25;
    }
    t->c = static_cast<float>(c);
    if (!std::isfinite(t->c)) return CSX_ERR_BAD_MODEL;
    for (int k = 0; k < kNtot; ++k) {
        t->lin[k] = static_cast<float>(lin[k]);
        if (!std::isfinite(t->lin[k])) return CSX_ERR_BAD_MODEL;
    }
    std::memset(t->btile, 0, sizeof(t->btile));
    for (int n = 0; n < 16; ++n)
        for (int k = 0; k < 16; ++k) {
            const float x = static_cast<float>(L[n][k] * scale);
            uint16_t bits;
            if (fp16) {
                const __half h = __float2half_rn(x);
                bits = *reinterpret_cast<const uint16_t *>(&h);
                if (!std::isfinite(__half2float(h))) return CSX_ERR_BAD_MODEL;
            } else {
                const __nv_bfloat16 h = __float2bfloat16_rn(x);
                bits = *reinterpret_cast<const uint16_t *>(&h);
                if (!std::isfinite(__bfloat162float(h))) return CSX_ERR_BAD_MODEL;
            }
            const int off = (n >> 3) * 256 + (k >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2;
            t->btile[off / 2] = bits;
        }
    t->tail = 0u;
    for (int k = 16; k < kNtot; ++k) t->tail |= m.w_lin[k] != 0.0f ? 1u : 0u;
    return CSX_OK;
}

// Bound on |precision-form score - exact score| for genes in [0, 1]
// (u = unit roundoff of the tile format, SL = sum |L_ij|, SL' = SL / 4):
//   BF16: x = bf16(g), L rounded: (2u + u^2) SL, u = 2^-9;
//   FP16: x' = fp16(fl(2g - 1)), L/4 rounded: (2u + u^2) SL' + 2^-25 (2 SL' + 136 * 2^-25)
//         (subnormal spacing and the f32 rounding of 2g - 1), u = 2^-12,
//         plus the f32 rounding of the folded constant and linear terms;
// and for both the tensor-core accumulation (taken as 2^-18 relative, a
// margin over FP32), the FP32 row dot (gamma_17) and the FP32 linear part
// (gamma_31) on the absolute sums of their terms.
int tc_error_bound(const csx_model &m, bool fp16, float *out) {
    double SL = 0.0, lin = 16.0 * std::fabs(static_cast<double>(m.w0));
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) SL += std::fabs(static_cast<double>(m.w_quad[i * 16 + j]));
    for (int k = 0; k < kNtot; ++k) lin += std::fabs(static_cast<double>(m.w_lin[k]));
    const double u24 = std::ldexp(1.0, -24);
    auto gamma = [u24](double n) { return n * u24 / (1.0 - n * u24); };
    double e;
    if (!fp16) {
        const double u = std::ldexp(1.0, -9);
        e = (2 * u + u * u) * SL + (std::ldexp(1.0, -18) + gamma(17)) * SL * (1 + 4 * u) + gamma(31) * lin;
    } else {
        const double u = std::ldexp(1.0, -12), sl = SL / 4.0;
        const double t25 = std::ldexp(1.0, -25);
        // folded terms: |c''| + sum |lin''| <= lin + 7 sl (u_i sums to 2 sl, v to sl)
        const double lin2 = lin + 7.0 * sl;
        e = (2 * u + u * u) * sl + t25 * (2 * sl + 136 * t25) + (std::ldexp(1.0, -18) + gamma(17)) * sl * 1.01 +
            (gamma(31) + u24) * lin2;
    }
    e = e * (1.0 + std::ldexp(1.0, -20)) + 1e-30;
    if (!std::isfinite(e) || e > 1e30) return CSX_ERR_BAD_MODEL;
    *out = std::nextafter(static_cast<float>(e), INFINITY);
    return CSX_OK;
}

// One 128-thread group scoring rows of a gene table (n x ldg floats).
template <bool kFp16>
__global__ void __launch_bounds__(128) tc_score_kernel(const __grid_constant__ TcModel M,
                                                       const float *__restrict__ genes, int64_t n, int ldg,
                                                       float *__restrict__ out, unsigned int *__restrict__ err) {
    __shared__ __align__(1024) unsigned char xs[4096];
    __shared__ __align__(16) uint16_t bt[256];
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ uint32_t tbase;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    for (uint32_t i = tid; i < 256; i += 128) bt[i] = M.btile[i];
    if (warp == 0) tc_alloc(smem_u32(&tbase), 32);
    if (tid == 0) mbar_init(smem_u32(&mbar), 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    TcGroup g;
    g.xs = smem_u32(xs);
    g.mbar = smem_u32(&mbar);
    g.tmem_d = tbase;
    g.tmem_ld = tbase + ((32u * (warp & 3u)) << 16);
    g.adesc = tc_sdesc(g.xs, 128, 256);
    g.bdesc = tc_sdesc(smem_u32(bt), 128, 256);
    g.idesc = tc_idesc(kFp16);
    g.bar_id = 1;
    g.phase = 0;
    g.issuer = tid == 0;
    bool ok = true;
    __shared__ uint32_t s_gbad, s_fail_phase;
    if (tid == 0) s_gbad = s_fail_phase = 0;
    __syncthreads();
    for (int64_t r0 = static_cast<int64_t>(blockIdx.x) * 128; r0 < n; r0 += static_cast<int64_t>(gridDim.x) * 128) {
        const int64_t r = r0 + tid;
        float x[16];
        float R = M.c;
        uint32_t pk[8];
#pragma unroll
        for (int k = 0; k < kNtot; ++k) {
            const float gk = (r < n) ? genes[r * ldg + k] : 0.0f;
            R = __fmaf_rn(M.lin[k], gk, R);
            if (k < 16) x[k] = kFp16 ? __fmaf_rn(gk, 2.0f, -1.0f) : gk;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) pk[j] = pack2(x[2 * j], x[2 * j + 1], kFp16);
        float y[16];
        if (!tcp_round(g, pk, tid, y, &s_gbad, &s_fail_phase)) ok = false;  // a give-up stops the MMAs
        float s = R;
#pragma unroll
        for (int i = 0; i < 16; ++i) s = __fmaf_rn(x[i], y[i], s);
        if (r < n) out[r] = s;
    }
    if (!ok) atomicOr(err, kErrTc);
    __syncthreads();
    if (s_gbad != 0u && g.issuer) (void)mbar_wait(g.mbar, s_fail_phase);  // bounded: the MMA given up on
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tc_dealloc(tbase, 32);
}

}  // namespace csx

extern "C" int csx_tc_score(const csx_model *model, int form, const float *d_genes, int64_t n, int ldg,
                            float *d_out, uint32_t *d_err, void *cuda_stream) {
    if (!model || (form != CSX_TC_BF16 && form != CSX_TC_FP16) || n < 0 || ldg < kNtot || !d_err) return CSX_ERR_BAD_ARGS;
    if (n > 0 && (!d_genes || !d_out)) return CSX_ERR_BAD_ARGS;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return CSX_ERR_NO_DEVICE;
    }
    const bool fp16 = form == CSX_TC_FP16;
    TcModel t;
    int rc = make_tc_model(*model, fp16, &t);
    if (rc) return rc;
    if (n == 0) return CSX_OK;
    int dev = 0, sms = 0;
    CSX_CUDA(cudaGetDevice(&dev));
    CSX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t tiles = (n + 127) / 128;
    const int grid = static_cast<int>(std::min<int64_t>(tiles, 8ll * sms));
    auto st = static_cast<cudaStream_t>(cuda_stream);
    if (fp16)
        tc_score_kernel<true><<<grid, 128, 0, st>>>(t, d_genes, n, ldg, d_out, reinterpret_cast<unsigned int *>(d_err));
    else
        tc_score_kernel<false><<<grid, 128, 0, st>>>(t, d_genes, n, ldg, d_out, reinterpret_cast<unsigned int *>(d_err));
    CSX_CUDA(cudaGetLastError());
    return CSX_OK;
}
