// csx_tc.cuh — tensor-core (tcgen05) scoring of the surrogate's quadratic
// block in BF16 or FP16, FP32 accumulation in tensor memory (sm_103a).
//
// The quadratic block of src/screen.zig:97-112 over the 16 legacy genes is
// sum_i x_i * (L x)_i with L lower-triangular (L_ij = Model.w_quad[i*16 + j]).
// 128 threads (four warps) each hold one candidate's genes; they write the
// rows x (bf16, or fp16 of x' = 2g - 1) into a shared-memory tile, one thread
// issues a single tcgen05.mma (M = 128, N = 16, K = 16) computing Y = X L^T
// into 16 columns of tensor memory, and each thread reads its own row back
// with tcgen05.ld (warp w of the group reads TMEM lanes 32(w % 4) ..). The
// rest of the score (constant, linear terms, and the row dot sum_i x_i y_i)
// is FP32 FMA on the thread's own values.
//
// Shared-memory tiles use the canonical no-swizzle K-major layout: core
// matrices of 8 rows x 16 bytes; element (r, k) at
//   (r / 8) * 256 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// so the descriptors carry LBO = 128 (next core matrix along K) and SBO = 256
// (next 8-row group).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>

namespace csx {

constexpr uint32_t kTcSpinLimit = 1u << 22;  // mbarrier polls before a wait gives up
constexpr uint32_t kErrTc = 16u;             // a tensor-core wait gave up (error bit)

// Precision form of a model: FP32 constant and linear terms on the exact
// genes, and the 16x16 B tile (L, or L/4 for the fp16 x' = 2g - 1 form) in
// the canonical layout above.
struct TcModel {
    float c;
    float lin[kNtot];
    alignas(16) uint16_t btile[256];
    uint32_t tail;  // some linear weight past gene 15 is nonzero (else genes 16..28 are skipped)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: start address, LBO and SBO in
// 16-byte units, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D = F32, A = B = BF16 (1) or F16 (0),
// both K-major, N = 16, M = 128.
__host__ __device__ constexpr uint32_t tc_idesc(bool fp16) {
    return (1u << 4) | ((fp16 ? 0u : 1u) << 7) | ((fp16 ? 0u : 1u) << 10) | ((16u >> 3) << 17) |
           ((128u >> 4) << 24);
}

__device__ __forceinline__ void tc_alloc(uint32_t dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with this parity; false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < kTcSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(0u)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&y)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) y[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack2(float a, float b, bool fp16) {
    if (fp16) {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const uint32_t *>(&h);
    }
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// One 128-thread group's shared state: X tile, mbarrier, TMEM columns.
struct TcGroup {
    uint32_t xs;      // shared address of the 4 KB X tile
    uint32_t mbar;    // shared address of the group's mbarrier
    uint32_t tmem_d;  // TMEM address of the group's 16 accumulator columns (lane 0)
    uint32_t tmem_ld; // this warp's lane quarter of those columns
    uint64_t adesc, bdesc;
    uint32_t idesc;
    uint32_t bar_id;  // named barrier of the group
    uint32_t phase;
    bool issuer;
};

// Row `row` (0..127) of the group's X tile <- packed x; one MMA for the group;
// y <- this thread's row of X L^T. All 128 threads of the group must call it.
// Returns false when the MMA's completion wait gave up (y is then garbage).
__device__ __forceinline__ bool tc_round(TcGroup &g, const uint32_t (&pk)[8], uint32_t row, float (&y)[16]) {
    const uint32_t a = g.xs + (row >> 3) * 256u + (row & 7u) * 16u;
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(pk[0]), "r"(pk[1]), "r"(pk[2]), "r"(pk[3])
                 : "memory");
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a + 128u), "r"(pk[4]), "r"(pk[5]), "r"(pk[6]),
                 "r"(pk[7])
                 : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    // literal barrier ids: a register id makes ptxas reserve all 16 named barriers,
    // which limits how many CTAs an SM holds
    if (g.bar_id == 1)
        asm volatile("bar.sync 1, 128;" ::: "memory");
    else
        asm volatile("bar.sync 2, 128;" ::: "memory");
    if (g.issuer) {
        tc_fence_after();
        tc_mma(g.tmem_d, g.adesc, g.bdesc, g.idesc);
        tc_commit(g.mbar);
    }
    const bool ok = mbar_wait(g.mbar, g.phase);
    g.phase ^= 1u;
    tc_fence_after();
    tc_ld16(g.tmem_ld, y);
    return ok;
}

}  // namespace csx

namespace csx {

// One candidate's genes exactly as synth_score makes them (src/screen.zig:
// 225-250; same draws, same rounding), consumed for the precision form:
// R = c + sum_k lin_k g_k (FP32 FMA), x = the 16 legacy genes (or 2g - 1 for
// FP16), pk = x packed in pairs for the tensor-core tile. The genes are the
// candidate's before its jump, as in synth_score's filter form.
template <bool kFastDelta, bool kFp16>
__device__ __forceinline__ void synth_tc(const TcModel &T, const SynthConst &C, const float *__restrict__ el,
                                         uint64_t seed_t, uint64_t p, const CandHead &h, float &R, float (&x)[16],
                                         uint32_t (&pk)[8]) {
    GeneSource S = gene_source(C, el, seed_t, p, h);
    R = T.c;
#pragma unroll
    for (int k = 0; k < kNtot; ++k) {
        if (k == 16 && !T.tail) break;  // no linear weight past gene 15: R gains +-0 from them
        const float g = next_gene<kFastDelta>(S, k);
        // no jump here: the caller lowers the threshold by JumpBound::c[h.jidx]
        R = __fmaf_rn(T.lin[k], g, R);
        if (k < 16) x[k] = kFp16 ? __fmaf_rn(g, 2.0f, -1.0f) : g;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) pk[j] = pack2(x[2 * j], x[2 * j + 1], kFp16);
}

// One tensor-core round of a 128-thread group (tc_round with a give-up path
// that keeps the group in step). gbad is the group's flag in
// shared memory, written only by the group's threads, after their wait of a
// round and before the next round's barrier: every thread of the group reads
// the same value after that barrier, so once a wait has given up the whole
// group skips the MMA and the wait from the next round on, and every thread
// still passes the same barriers. *fail_phase receives the parity of the
// wait that gave up. Returns false when this thread's wait gave up.
__device__ __forceinline__ bool tcp_round(TcGroup &g, const uint32_t (&pk)[8], uint32_t row, float (&y)[16],
                                          volatile uint32_t *gbad, volatile uint32_t *fail_phase) {
    const uint32_t a = g.xs + (row >> 3) * 256u + (row & 7u) * 16u;
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(pk[0]), "r"(pk[1]), "r"(pk[2]), "r"(pk[3])
                 : "memory");
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a + 128u), "r"(pk[4]), "r"(pk[5]), "r"(pk[6]),
                 "r"(pk[7])
                 : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    if (g.bar_id == 1)
        asm volatile("bar.sync 1, 128;" ::: "memory");
    else
        asm volatile("bar.sync 2, 128;" ::: "memory");
    if (*gbad != 0u) {
#pragma unroll
        for (int i = 0; i < 16; ++i) y[i] = 0.0f;
        return true;
    }
    if (g.issuer) {
        tc_fence_after();
        tc_mma(g.tmem_d, g.adesc, g.bdesc, g.idesc);
        tc_commit(g.mbar);
    }
    const bool ok = mbar_wait(g.mbar, g.phase);
    if (!ok) {
        *fail_phase = g.phase;
        *gbad = 1u;
    }
    g.phase ^= 1u;
    tc_fence_after();
    tc_ld16(g.tmem_ld, y);
    return ok;
}

}  // namespace csx
