// csx_device.cuh — device primitives of the screen funnel (sm_103a).
//
// One candidate of src/screen.zig:225-253 is synthesised and scored per call,
// entirely in registers. splitmix64 (src/screen.zig:202-208) is counter based:
// the state before draw q of stream t is seed_t + q*G, so any draw can be
// computed directly from its position. Every use below computes only the
// part of the 64-bit output it consumes:
//   * parent / jump index   (next() >> 32):  hi word, final xor-shift kept
//   * unit()  (next() >> 40): bits 63..40 are untouched by the final
//     `z ^ (z >> 31)`, so the hi word of the second product suffices
//   * crossover bit (next() & 1) = bit0 ^ bit31 of the low word of the second
//     product; multiplying that low word by (2^31 + 1) moves the XOR into bit
//     31, and the factor folds into the multiply constant: one IMUL.
// All f32 arithmetic that reaches a gene or a score uses explicit _rn
// intrinsics, so nothing is contracted into FMA unless written as one.
#pragma once

#include <cstdint>

namespace csx {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;
constexpr uint64_t kMix1 = 0xBF58476D1CE4E5B9ull;
constexpr uint64_t kMix2 = 0x94D049BB133111EBull;
constexpr uint32_t kMix2LoFold = static_cast<uint32_t>(kMix2) * 0x80000001u;
constexpr int kNtot = 29;
constexpr int kNq = 136;  // lower-triangular quad terms over the 16 legacy genes

// Model in the compact triangular form used on the device.
// The full quadratic surface over all 29 genes (no reference code: the
// extension docs/RESEARCH_V05C.md:99-102 queues). Its f32 score is defined
// by one FMA order, r = w0; t_k = fma chain of w_lin[k] + sum_{l<=k} Q_kl g_l;
// r = fma(g_k, t_k, r) for k = 0..28 -- the order synth_full evaluates while
// the genes are synthesised, and the oracle's orc_score_full.
constexpr int kNqFull = kNtot * (kNtot + 1) / 2;  // 435
struct FullModel {
    float w0;
    float wlin[kNtot];
    float wq[kNqFull];  // (i, j <= i) at i*(i+1)/2 + j
};

struct DevModel {
    float w0;
    float w16;  // 16 * w0 (exact): the intercept as Model.score counts it
    float wlin[kNtot];
    float wq[kNq];  // (i, j <= i) at i*(i+1)/2 + j  ==  Model.w_quad[i*16 + j]
    uint32_t tail;  // some linear weight past gene 15 is nonzero (synth_score)
};

// Bound on how far a jump can raise the real score: with every gene in
// [0, 1], setting gene j to another value in [0, 1] raises the surface by at
// most c[j] (host: jump_bound, from the signs of w_lin[j] and gene j's
// quadratic terms; rounded up). c[kNoJump] = 0, as are the unused entries.
struct JumpBound {
    float c[32];
};

// Per-call synthesis constants (uniform across the grid).
struct SynthConst {
    uint64_t ne_magic;  // Lemire fastmod constant for ne
    uint32_t ne;        // elite count; row ne of the elite table holds 0.5s
    uint32_t imm_thr;   // unit() < imm_p   <=>  (next() >> 40) < imm_thr
    uint32_t jump_thr;  // unit() < jump_p  <=>  (next() >> 40) < jump_thr
    float sigma;
    float nsig1;    // -sigma
    float sigma23;  // sigma * 2^-23 (exact in the fast delta form)
};

__host__ __device__ constexpr int tri(int i, int j) { return i * (i + 1) / 2 + j; }

// The same coefficients in the order synth_score's filter form consumes them,
// each gene's group starting on 16 bytes so that a shared-memory copy is read
// with 16-byte loads: row k < 16 holds Wq[k][0..k] then w_lin[k]; then
// w_lin[16..28]; then w16 and w0.
__host__ __device__ constexpr int row_off(int k) {
    int o = 0;
    for (int j = 0; j < k; ++j) o += ((j + 2 + 3) / 4) * 4;
    return o;
}
constexpr int kRowLin16 = row_off(16);      // 176
constexpr int kRowW16 = kRowLin16 + 16;     // 192: w16, w0, then the tail flag (1.0f / 0.0f)
constexpr int kRowModelFloats = kRowW16 + 4;

struct alignas(16) RowModel {
    float v[kRowModelFloats];
};

// Coefficient access for synth_score: kernel-parameter DevModel or RowModel.
__device__ __forceinline__ float m_q(const DevModel &M, int k, int l) { return M.wq[tri(k, l)]; }
__device__ __forceinline__ float m_lin(const DevModel &M, int k) { return M.wlin[k]; }
__device__ __forceinline__ float m_w0(const DevModel &M) { return M.w0; }
__device__ __forceinline__ float m_w16(const DevModel &M) { return M.w16; }
__device__ __forceinline__ float m_q(const RowModel &M, int k, int l) { return M.v[row_off(k) + l]; }
__device__ __forceinline__ float m_lin(const RowModel &M, int k) {
    return k < 16 ? M.v[row_off(k) + k + 1] : M.v[kRowLin16 + k - 16];
}
__device__ __forceinline__ float m_w0(const RowModel &M) { return M.v[kRowW16 + 1]; }
__device__ __forceinline__ float m_w16(const RowModel &M) { return M.v[kRowW16]; }
__device__ __forceinline__ bool m_tail(const DevModel &M) { return M.tail != 0u; }
__device__ __forceinline__ bool m_tail(const RowModel &M) { return M.v[kRowW16 + 2] != 0.0f; }

// y = z * kMix1 where z = s ^ (s >> 30): the first half of the mixer.
__device__ __forceinline__ uint64_t mix_a(uint64_t s) {
    const uint64_t z = s ^ (s >> 30);
    return z * kMix1;
}

// hi word of v = u * kMix2, u = y ^ (y >> 27). Bits 31..8 of it are bits
// 63..40 of next(); (vh >> 8) is next() >> 40.
__device__ __forceinline__ uint32_t draw_vh(uint64_t s) {
    const uint64_t y = mix_a(s);
    const uint64_t u = y ^ (y >> 27);
    return static_cast<uint32_t>((u * kMix2) >> 32);
}

// next() >> 32.
__device__ __forceinline__ uint32_t draw_hi(uint64_t s) {
    const uint32_t vh = draw_vh(s);
    return vh ^ (vh >> 31);
}

// Sign bit == next() & 1.
__device__ __forceinline__ uint32_t draw_bitword(uint64_t s) {
    const uint64_t y = mix_a(s);
    const uint32_t ul = static_cast<uint32_t>(y ^ (y >> 27));
    return ul * kMix2LoFold;
}

// x % d for 32-bit x and 1 <= d < 2^32 (Lemire, Kaser, Kurz 2019):
// M = floor((2^64 - 1) / d) + 1, x % d = hi64((M * x mod 2^64) * d).
__device__ __forceinline__ uint32_t fastmod_u32(uint32_t x, uint64_t M, uint32_t d) {
    const uint64_t low = M * x;
    const uint32_t lo = static_cast<uint32_t>(low), hi = static_cast<uint32_t>(low >> 32);
    const uint64_t p1 = static_cast<uint64_t>(hi) * d + __umulhi(lo, d);
    return static_cast<uint32_t>(p1 >> 32);
}

// Header of the candidate at draw position p (src/screen.zig:232-235,247-248).
// A candidate without a jump carries jidx = kNoJump, past the last gene, so
// that a 32-entry per-gene table (JumpBound) is indexed without a test.
constexpr uint32_t kNoJump = 31;
struct CandHead {
    uint32_t ea, eb;   // parent rows
    uint32_t jidx;     // jump gene index, kNoJump when no jump
    float jval;        // jump value
    bool imm;          // immigrant
    uint32_t len;      // draws the candidate consumes: 33/35/62/64
};

__device__ __forceinline__ CandHead cand_head(const SynthConst &C, uint64_t seed_t, uint64_t p) {
    CandHead h;
    const uint64_t s0 = seed_t + (p + 1) * kGolden;  // state after draw p's increment
    h.ea = fastmod_u32(draw_hi(s0), C.ne_magic, C.ne);
    h.eb = fastmod_u32(draw_hi(s0 + kGolden), C.ne_magic, C.ne);
    h.imm = (draw_vh(s0 + 2 * kGolden) >> 8) < C.imm_thr;
    const uint64_t sj = s0 + (h.imm ? 32ull : 61ull) * kGolden;  // draw p+3+29 / p+3+58
    const bool jump = (draw_vh(sj) >> 8) < C.jump_thr;
    // the index (drawn first) and value only for the 2% that jump
    h.jidx = kNoJump;
    h.jval = 0.0f;
    if (jump) {
        h.jidx = draw_hi(sj + kGolden) % 29u;
        h.jval = static_cast<float>(draw_vh(sj + 2 * kGolden) >> 8) * (1.0f / 16777216.0f);
    }
    h.len = (h.imm ? 33u : 62u) + (jump ? 2u : 0u);
    return h;
}

// Synthesis state of one candidate (src/screen.zig:236-246): the parent rows
// (row ne, all 0.5, for an immigrant), the mutation constants (an immigrant's
// 0.5 + (u - 0.5) = u draws its genes uniformly) and the splitmix64 state of
// gene 0's unit draw; a crossover gene's bit draw precedes its unit draw.
struct GeneSource {
    const float *pa, *pb;
    float B, nb1, B23;
    uint64_t su, step;
};

__device__ __forceinline__ GeneSource gene_source(const SynthConst &C, const float *__restrict__ el,
                                                  uint64_t seed_t, uint64_t p, const CandHead &h) {
    GeneSource S;
    const uint64_t s0 = seed_t + (p + 1) * kGolden;
    S.pa = el + (h.imm ? C.ne : h.ea) * kNtot;
    S.pb = el + (h.imm ? C.ne : h.eb) * kNtot;
    S.B = h.imm ? 0.5f : C.sigma;
    S.nb1 = h.imm ? -0.5f : C.nsig1;
    S.B23 = h.imm ? 0x1p-24f : C.sigma23;
    S.step = h.imm ? kGolden : 2 * kGolden;
    S.su = s0 + (h.imm ? 3ull : 4ull) * kGolden;
    return S;
}

// Gene k before the jump: crossover parent, mutation, clamp01 (NaN -> 1, as
// @min(1, NaN) == 1; the fast form's delta is finite and the elite table holds
// no NaN, so g is never NaN there). Advances S to the next gene's draws.
template <bool kFastDelta>
__device__ __forceinline__ float next_gene(GeneSource &S, int k) {
    const uint32_t bw = draw_bitword(S.su - kGolden);  // crossover bit draw
    const uint32_t vh = draw_vh(S.su);                 // unit draw
    S.su += S.step;
    const float *src = (static_cast<int32_t>(bw) < 0) ? S.pb : S.pa;
    const float par = src[k];
    float g;
    if (kFastDelta) {
        g = __fadd_rn(par, __fmaf_rn(__uint2float_rn(vh >> 8), S.B23, S.nb1));
        g = fmaxf(fminf(g, 1.0f), 0.0f);
    } else {
        const float y = __uint_as_float(((vh >> 8) & 0x7FFFFFu) | 0x3F800000u);
        const float nc = (static_cast<int32_t>(vh) < 0) ? -1.0f : -2.0f;
        g = __fadd_rn(par, __fmul_rn(__fadd_rn(y, nc), S.B));
        g = (g != g) ? 1.0f : fmaxf(fminf(g, 1.0f), 0.0f);
    }
    return g;
}

// One candidate: genes in registers, score in the reference's op order
// (src/screen.zig:97-112):
//   lane l:  acc_l = w0 + wl_l*g_l;  sum_l = sum_{i=l..15} Wq[i][l]*(g_l*g_i)
//   score = (((acc_0+sum_0) + (acc_1+sum_1)) + ... ) + rsum,  rsum = sum_{k>=16} wl_k*g_k
// The strict upper triangle of Wq is +0 and g >= 0, so its terms add +0 and
// are skipped; the first add into sum_l keeps the reference's 0 + x.
//
// Immigrants (src/screen.zig:235-237) run the crossover arithmetic with both
// parents on a row of 0.5s and half-width 0.5: 0.5 + (u - 0.5) == u exactly.
// Their unit draws are consecutive; crossover genes alternate bit and unit.
//
// kFastDelta: (u - 0.5) * 2 = k * 2^-23 - 1 with k = next() >> 40, so the
// mutation round((u - 0.5) * 2 * B) is one FFMA, fma(float(k), B * 2^-23, -B):
// float(k) (24 bits), B * 2^-23 and -B are exact and the FFMA rounds once.
// Valid for B = 0 or 1e-30 <= |B| <= 1e38 (B * 2^-23 stays normal, |delta|
// < |B| stays finite); otherwise the two-op form builds u - 0.5 exactly from
// the mantissa bits and multiplies.
//
// kExact = false computes a filter score instead: the same surface by FFMA
// Horner, t_l = w_l + sum_{i>=l} Wq[i][l] g_i, s = 16 w0 + sum_l g_l t_l +
// sum_{k>=16} w_k g_k (165 FFMA). Both orders are within gamma_n * A of the
// real value (A = sum of |terms|), so the host bounds |fast - exact| and the
// exact order is evaluated only for candidates the bound cannot rule out.
// The filter form leaves the jump out (one compare and select per gene for
// 2% of candidates): replacing gene j moves the real score by at most
// JumpBound::c[j], which the caller adds to the bound.
// kJump: apply the jump (the exact form and kept genes always do; the filter
// form leaves it out unless asked, as described above).
// kScoreOnly (the default without kept genes): for a surface whose linear
// weights past gene 15 are all +-0 (m_tail false), genes 16..28 are not
// synthesised (their 26 draws skipped): each of their terms is +-0 times a
// finite gene, the tail sum starts from +0 and so stays +0, and the score is
// the lanes' sum + 0 either way. The jump's draws sit at fixed offsets from
// the candidate's start (cand_head), so it applies as before. With kept genes
// and kScoreOnly, genes[16..28] are left as the caller set them.
template <bool kFastDelta, bool kKeepGenes, bool kExact = true, class Model = DevModel,
          bool kJump = kExact || kKeepGenes, bool kScoreOnly = !kKeepGenes>
__device__ __forceinline__ float synth_score(const Model &M, const SynthConst &C,
                                             const float *__restrict__ el, uint64_t seed_t,
                                             uint64_t p, const CandHead &h, float *genes) {
    const bool tail = !kScoreOnly || m_tail(M);
    // next_gene's synthesis written out: through the helper the compiler
    // allocates this hot loop's registers differently (0.3% slower, measured)
    const uint64_t s0 = seed_t + (p + 1) * kGolden;
    const uint32_t ra = h.imm ? C.ne : h.ea;
    const uint32_t rb = h.imm ? C.ne : h.eb;
    const float *pa = el + ra * kNtot;
    const float *pb = el + rb * kNtot;
    const float B = h.imm ? 0.5f : C.sigma;
    const float nb1 = h.imm ? -0.5f : C.nsig1;
    const float B23 = h.imm ? 0x1p-24f : C.sigma23;
    const uint64_t step = h.imm ? kGolden : 2 * kGolden;
    uint64_t su = s0 + (h.imm ? 3ull : 4ull) * kGolden;  // unit draw of gene 0

    float G[16], S[16];
    float R = kExact ? 0.0f : m_w16(M);
#pragma unroll
    for (int k = 0; k < kNtot; ++k) {
        if (k == 16 && !tail) break;  // warp-uniform: one surface per call
        const uint32_t bw = draw_bitword(su - kGolden);  // crossover bit draw
        const uint32_t vh = draw_vh(su);                 // unit draw
        su += step;
        const float *src = (static_cast<int32_t>(bw) < 0) ? pb : pa;
        const float par = src[k];
        float g;
        if (kFastDelta) {
            g = __fadd_rn(par, __fmaf_rn(__uint2float_rn(vh >> 8), B23, nb1));
        } else {
            const float y = __uint_as_float(((vh >> 8) & 0x7FFFFFu) | 0x3F800000u);
            const float nc = (static_cast<int32_t>(vh) < 0) ? -1.0f : -2.0f;
            g = __fadd_rn(par, __fmul_rn(__fadd_rn(y, nc), B));
        }
        // clamp01 (NaN -> 1, as @min(1, NaN) == 1). The fast form's delta is
        // finite and the elite table holds no NaN, so g is never NaN there.
        if (kFastDelta)
            g = fmaxf(fminf(g, 1.0f), 0.0f);
        else
            g = (g != g) ? 1.0f : fmaxf(fminf(g, 1.0f), 0.0f);
        // The filter form scores the genome before the jump; the caller
        // widens its threshold by JumpBound::c[h.jidx] instead.
        if (kJump) g = (static_cast<uint32_t>(k) == h.jidx) ? h.jval : g;
        if (kKeepGenes) genes[k] = g;
        if (!kExact) {
            if (k < 16) {
                G[k] = g;
#pragma unroll
                for (int l = 0; l < k; ++l) S[l] = __fmaf_rn(m_q(M, k, l), g, S[l]);
                S[k] = __fmaf_rn(m_q(M, k, k), g, m_lin(M, k));
            } else {
                R = __fmaf_rn(m_lin(M, k), g, R);
            }
        } else if (k < 16) {
            G[k] = g;
#pragma unroll
            for (int l = 0; l < k; ++l)
                S[l] = __fadd_rn(S[l], __fmul_rn(m_q(M, k, l), __fmul_rn(G[l], g)));
            S[k] = __fadd_rn(0.0f, __fmul_rn(m_q(M, k, k), __fmul_rn(g, g)));
        } else {
            const float t = __fmul_rn(m_lin(M, k), g);
            R = (k == 16) ? __fadd_rn(0.0f, t) : __fadd_rn(R, t);
        }
    }
    if (!kExact) {
#pragma unroll
        for (int l = 0; l < 16; ++l) R = __fmaf_rn(G[l], S[l], R);
        return R;
    }
    float r = __fadd_rn(__fadd_rn(m_w0(M), __fmul_rn(m_lin(M, 0), G[0])), S[0]);
#pragma unroll
    for (int l = 1; l < 16; ++l)
        r = __fadd_rn(r, __fadd_rn(__fadd_rn(m_w0(M), __fmul_rn(m_lin(M, l), G[l])), S[l]));
    return __fadd_rn(r, R);
}

// One candidate scored on the full surface (FullModel's FMA order), the
// synthesis exactly as synth_score's: genes in registers, the jump applied.
template <bool kFastDelta, bool kKeepGenes>
__device__ __forceinline__ float synth_full(const FullModel &M, const SynthConst &C,
                                            const float *__restrict__ el, uint64_t seed_t, uint64_t p,
                                            const CandHead &h, float *genes) {
    GeneSource S = gene_source(C, el, seed_t, p, h);

    float G[kNtot];
    float R = M.w0;
#pragma unroll
    for (int k = 0; k < kNtot; ++k) {
        float g = next_gene<kFastDelta>(S, k);
        g = (static_cast<uint32_t>(k) == h.jidx) ? h.jval : g;
        if (kKeepGenes) genes[k] = g;
        G[k] = g;
        float t = M.wlin[k];
#pragma unroll
        for (int l = 0; l <= k; ++l) t = __fmaf_rn(M.wq[tri(k, l)], G[l], t);
        R = __fmaf_rn(g, t, R);
    }
    return R;
}

// The full surface's score of given genes, in synth_full's order.
__device__ __forceinline__ float score_full(const FullModel &M, const float (&g)[kNtot]) {
    float R = M.w0;
#pragma unroll
    for (int k = 0; k < kNtot; ++k) {
        float t = M.wlin[k];
#pragma unroll
        for (int l = 0; l <= k; ++l) t = __fmaf_rn(M.wq[tri(k, l)], g[l], t);
        R = __fmaf_rn(g[k], t, R);
    }
    return R;
}

// Model.score (src/screen.zig:97-112) of given genes, in the same f32 order as
// synth_score's exact form: lane l holds w0 + wl_l g_l + sum_{i>=l} Wq[i][l]
// (g_l g_i) accumulated row by row, the lanes are summed in order, then the
// tail sum_{k>=16} wl_k g_k is added.
__device__ __forceinline__ float score_genes_exact(const DevModel &M, const float (&g)[kNtot]) {
    float S[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
#pragma unroll
        for (int l = 0; l < k; ++l) S[l] = __fadd_rn(S[l], __fmul_rn(M.wq[tri(k, l)], __fmul_rn(g[l], g[k])));
        S[k] = __fadd_rn(0.0f, __fmul_rn(M.wq[tri(k, k)], __fmul_rn(g[k], g[k])));
    }
    float R = 0.0f;
#pragma unroll
    for (int k = 16; k < kNtot; ++k) {
        const float t = __fmul_rn(M.wlin[k], g[k]);
        R = (k == 16) ? __fadd_rn(0.0f, t) : __fadd_rn(R, t);
    }
    float r = __fadd_rn(__fadd_rn(M.w0, __fmul_rn(M.wlin[0], g[0])), S[0]);
#pragma unroll
    for (int l = 1; l < 16; ++l) r = __fadd_rn(r, __fadd_rn(__fadd_rn(M.w0, __fmul_rn(M.wlin[l], g[l])), S[l]));
    return __fadd_rn(r, R);
}

// Length of the candidate whose start draw has state st = seed_t + (p + 1) *
// kGolden: the immigrant test and the crossover candidate's jump test hashed
// side by side, the immigrant's own jump test only when it is one.
__device__ __forceinline__ uint32_t cand_len(const SynthConst &C, uint64_t st) {
    const uint32_t vi = draw_vh(st + 2 * kGolden);
    const uint32_t vj = draw_vh(st + 61 * kGolden);
    uint32_t len = 62;
    bool jump = (vj >> 8) < C.jump_thr;
    if ((vi >> 8) < C.imm_thr) {
        len = 33;
        jump = (draw_vh(st + 32 * kGolden) >> 8) < C.jump_thr;
    }
    return len + (jump ? 2u : 0u);
}

// Order-preserving key of a score; -0 ranks with +0 and NaN below everything.
__device__ __forceinline__ uint32_t score_okey(float x) {
    x = __fadd_rn(x, 0.0f);
    const uint32_t b = __float_as_uint(x);
    const uint32_t k = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    return (x != x) ? 0u : k;
}

__device__ __forceinline__ float okey_score(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

}  // namespace csx
