// csx_prune.cuh — the pruning screen: a certified upper bound of each
// candidate's score from its parents and crossover bits, taken before its
// mutation draws, so that a candidate which cannot reach the top-K skips them.
// Part of csx_screen.cu's translation unit (included there, in order); not a
// standalone header.
//
// The reference scores every candidate in full (src/screen.zig:225-253: two
// parent draws, the immigrant test, 29 x (crossover bit + mutation unit), the
// jump test, Model.score). Here a crossover candidate costs four header draws
// and the crossover bits of the genes the surface reads (16 for the 153 / 161
// layouts, whose linear weights past gene 15 are zero; 29 otherwise), plus the
// bound below; only candidates the bound cannot rule out, and immigrants, are
// synthesised in full and scored in the reference's f32 order (the queue of
// the filter form). The survivors, their scores and the screened count are
// those of the reference's run: a candidate is skipped only when its score is
// certainly below the K-th score of candidates already screened.
//
// The bound. Gene k of a crossover candidate is g_k = clamp01(par_k + d_k)
// with par_k the parent's gene chosen by the crossover bit and |d_k| <=
// |sigma|; with y_k = clamp01(par_k), |g_k - y_k| <= s = min(|sigma| + 2^-24,
// 1) (clamp01 is monotone and 1-Lipschitz; 2^-24 covers the rounding of
// par_k + d_k where it is not clamped). The surface is the quadratic
//   f(g) = 16 w0 + sum_k w_k g_k + sum_{j<=i<16} Q_ij g_i g_j,
// so with u = g - y:
//   f(g) = f(y) + grad f(y) . u + sum_{j<=i<16} Q_ij u_i u_j
//        <= f(y) + s sum_k |grad_k f(y)| + c0,
//   c0 = s sum_{k>=16} |w_k| + s^2 (sum_i max(Q_ii, 0) + sum_{j<i} |Q_ij|).
// grad f(y) = w + Qs y over the first 16 genes (Qs = Q + Q^T) and w_k past
// them; f(y) = 16 w0 + sum_k y_k (w_k + grad_k) / 2 + sum_{k>=16} w_k y_k.
// A jump replaces one gene by a value in [0, 1], which raises f by at most
// JumpBound::c[j]. The bound is evaluated in f32; PruneConst::err covers its
// rounding and the reference order's (a candidate's f32 score is within
// gamma_35 * A of its real value), so a candidate is skipped only when
//   bound + err + c[j] < K-th score.
#pragma once

namespace csx {

constexpr int kPruneMs = 3;  // order statistics each CTA publishes: its 1st, 2nd and 4th best
constexpr uint32_t kPruneMergeRounds = 16;  // rounds between merges of a non-empty buffer

struct PruneConst {
    float qs[16][16];  // Qs = Q + Q^T (Qs_kk = 2 Q_kk): grad of the quadratic block is Qs y
    float s;           // half-width of a gene's mutation box around clamp01(parent gene)
    float c0;          // the bound's constant part (above), rounded up
    float err;         // bound rounding + reference-order rounding, rounded up
};

// The bound's gradient on the tensor cores: Qs * 2^-e in FP16 (e chosen so
// that the largest entry is near 2^15), the canonical no-swizzle K-major tile
// of csx_tc.cuh; the MMA gives D = Yh Qh with Yh the FP16 parent genes, and
// grad = wl + 2^e D within PruneTc::err's share (see make_prune_tc). The
// bound is centred on yh = fp16(y) itself (|yh - y| <= 2^-12 widens the box),
// so the thread needs only the packed FP16 genes it hands to the MMA.
struct PruneTc {
    alignas(16) uint16_t btile[256];
    float dscale;  // 2^e
    float s;       // half-width around the FP16 centre: PruneConst::s + 2^-12, rounded up
    float c0;      // PruneConst::c0 at that half-width
    float err;     // replaces PruneConst::err in this form
};

struct PruneArgs : ScreenArgs {
    PruneConst pc;
    PruneTc tc;
    uint32_t *pub;     // kPruneMs x gridDim.x: okey of each CTA's 1st / 2nd / 4th best entry
    uint32_t sel_cap;  // entries of the selection scratch in shared memory (>= gridDim.x)
    uint32_t el_smem;  // 1: the elite table is copied to shared memory (prune_el_smem)
};

// Row stride of the clamped parent table: odd, so that a warp reading random
// rows at one gene spreads over the banks.
template <int kNb>
constexpr int prune_stride() {
    return kNb == 16 ? 17 : kNtot;
}

// Header of a candidate for the pruning form: parents, immigrant test, jump
// test and the jump gene index (not its value), and the candidate's length.
struct PruneHead {
    uint32_t ea, eb, jidx, len;
    bool imm;
};

__device__ __forceinline__ PruneHead prune_head(const SynthConst &C, uint64_t s0) {
    PruneHead h;
    h.ea = fastmod_u32(draw_hi(s0), C.ne_magic, C.ne);
    h.eb = fastmod_u32(draw_hi(s0 + kGolden), C.ne_magic, C.ne);
    h.imm = (draw_vh(s0 + 2 * kGolden) >> 8) < C.imm_thr;
    const uint64_t sj = s0 + (h.imm ? 32ull : 61ull) * kGolden;
    const bool jump = (draw_vh(sj) >> 8) < C.jump_thr;
    h.jidx = kNoJump;
    if (jump) h.jidx = draw_hi(sj + kGolden) % 29u;
    h.len = (h.imm ? 33u : 62u) + (jump ? 2u : 0u);
    return h;
}

// The bound of the crossover candidate whose first draw has state s0 (before
// its jump), parents ea / eb; yt is the clamped parent table.
template <int kNb>
__device__ __forceinline__ float prune_bound(const PruneArgs &A, const float *__restrict__ yt, uint64_t s0,
                                             uint32_t ea, uint32_t eb) {
    constexpr int kYs = prune_stride<kNb>();
    const float *ya = yt + ea * kYs;
    const float *yb = yt + eb * kYs;
    uint64_t sb = s0 + 3 * kGolden;  // crossover bit draw of gene 0
    float g[16], y[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) g[j] = A.m.wlin[j];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const uint32_t bw = draw_bitword(sb);
        sb += 2 * kGolden;
        y[k] = ((static_cast<int32_t>(bw) < 0) ? yb : ya)[k];
#pragma unroll
        for (int j = 0; j < 16; ++j) g[j] = __fmaf_rn(A.pc.qs[j][k], y[k], g[j]);
    }
    float f2 = 0.0f, l1 = 0.0f;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        f2 = __fmaf_rn(y[k], __fadd_rn(g[k], A.m.wlin[k]), f2);
        l1 = __fadd_rn(l1, fabsf(g[k]));
    }
    float r = __fmaf_rn(0.5f, f2, A.m.w16);
    if (kNb > 16) {
#pragma unroll
        for (int k = 16; k < kNb; ++k) {
            const uint32_t bw = draw_bitword(sb);
            sb += 2 * kGolden;
            r = __fmaf_rn(A.m.wlin[k], ((static_cast<int32_t>(bw) < 0) ? yb : ya)[k], r);
        }
    }
    return __fadd_rn(__fmaf_rn(A.pc.s, l1, r), A.pc.c0);
}

// FP64 score of a queued candidate for the precision form, out of line. Its
// full synthesis, jump applied, is scored by the FFMA filter first (within
// ScreenArgs::err of the real score); only a candidate the filter cannot
// place below tlo = threshold - err is scored in FP64 (rounded to f32, which
// err covers as well): the FP64 pipe runs at a small fraction of the FP32
// rate. A filtered-out candidate returns -inf.
__device__ __noinline__ float prune_rescore64(const ScreenArgs *__restrict__ A, const float *el, uint64_t seed_t,
                                              uint64_t p, float tlo) {
    const CandHead h = cand_head(A->sc, seed_t, p);
    const float sf = synth_score<true, false, false, DevModel, true>(A->m, A->sc, el, seed_t, p, h, nullptr);
    if (sf < tlo) return -INFINITY;
    return static_cast<float>(score64_at<true>(&A->m, &A->sc, el, seed_t, p));  // out of line: own registers
}

// Score of a queued candidate: the reference's f32 order (out of line), or
// the precision form's FP64 score.
template <bool kFp64>
__device__ __forceinline__ float prune_rescore(const ScreenArgs *__restrict__ A, const float *el, uint64_t seed_t,
                                               uint64_t p, float tlo) {
    if (!kFp64) return exact_score_at<true>(A, el, seed_t, p);
    return prune_rescore64(A, el, seed_t, p, tlo);
}

// The j-th largest (1-based) of v[0..n), by one warp (every lane calls):
// bisection on the 32-bit key, the largest x with #{v >= x} >= j.
__device__ __forceinline__ uint32_t warp_kth_largest(const uint32_t *v, uint32_t n, uint32_t j) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t prefix = 0;
    for (int b = 31; b >= 0; --b) {
        const uint32_t cand = prefix | (1u << b);
        uint32_t c = 0;
        for (uint32_t i = lane; i < n; i += 32) c += (v[i] >= cand) ? 1u : 0u;
        c = __reduce_add_sync(0xffffffffu, c);
        if (c >= j) prefix = cand;
    }
    return prefix;
}

// The pruning screen (persistent, dynamic items, the filter form's queue).
// Global threshold: besides the best CTA K-th score (Ctrl::gtau), every CTA
// publishes the keys of its m-th best entry, m = 1, 2, 4. If ceil(K / m) CTAs
// have published keys >= x, at least K distinct screened candidates score at
// least x, so the generation's K-th score is >= x; each published key only
// grows, so a stale read gives a lower, still valid, threshold. After each
// merge warp 0 takes the best such x and raises Ctrl::gtau to it.
template <int kNb>
__global__ void __launch_bounds__(kThreads, 2) screen_p_kernel(const __grid_constant__ PruneArgs A) {
    constexpr int kYs = prune_stride<kNb>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Entry *E = reinterpret_cast<Entry *>(smem_raw);
    // the elite table: only the queued candidates' full synthesis reads it;
    // in shared memory where that costs no CTA per SM, else through L1
    float *el_copy = reinterpret_cast<float *>(E + A.sort_n);
    const float *el = A.el_smem ? el_copy : A.el;
    Pend *pend = reinterpret_cast<Pend *>(el_copy + (A.el_smem ? (A.sc.ne + 1) * kNtot : 0u));
    float *yt = reinterpret_cast<float *>(pend + kPendCap);
    uint32_t *sel = reinterpret_cast<uint32_t *>(yt + A.sc.ne * kYs);
    __shared__ unsigned int s_buf_n, s_pend_n;
    __shared__ unsigned long long s_t1, s_t2;
    __shared__ float s_ts;

    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i < A.sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
    if (A.el_smem)
        for (uint32_t i = tid; i < (A.sc.ne + 1) * kNtot; i += kThreads) el_copy[i] = A.el[i];
    for (uint32_t i = tid; i < A.sc.ne * kYs; i += kThreads) {
        const uint32_t r = i / kYs, k = i - r * kYs;
        // +inf (a NaN elite gene) clamps to 1, as the reference's clamp01(NaN + d)
        yt[i] = (k < static_cast<uint32_t>(kNb)) ? fmaxf(fminf(A.el[r * kNtot + k], 1.0f), 0.0f) : 0.0f;
    }
    if (tid == 0) {
        s_buf_n = 0;
        s_pend_n = 0;
        s_t1 = 0;
        s_t2 = 0;
        s_ts = -INFINITY;
    }
    const unsigned int n_items = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->n_items);
    __syncthreads();

    Entry *buf = E + A.kpad;
    uint32_t item = atomicAdd(&A.ctrl->next_item, 1u);
    bool valid = item < n_items;
    uint64_t seed_t = 0, p = 0;
    uint32_t left = 0, dcand = 0, ddraw = 0;
    if (valid) {
        const Item it = A.items[item];
        seed_t = stream_seed(A.seed, it.stream);
        p = it.draw0;
        left = it.n;
        valid = left > 0;
    }
    unsigned long long screened = 0, exact = 0;
    unsigned int gk = 0;
    uint32_t round = 0;
    bool has_def = false;  // holds a candidate the full queue could not take; pauses until the merge
    Pend def{0u, 0u, 0u};

    auto rescore = [&](const Pend &q, unsigned long long t1, unsigned long long t2, float ts) {
        const Item it = A.items[q.item];
        const float s = exact_score_at<true>(&A, el, stream_seed(A.seed, it.stream), it.draw0 + q.ddraw);
        ++exact;
        if (s >= ts) {
            const unsigned long long k1 =
                (static_cast<unsigned long long>(score_okey(s)) << 32) | static_cast<unsigned int>(~q.item);
            const unsigned long long k2 = (static_cast<unsigned long long>(~q.dcand) << 32) | q.ddraw;
            buf[atomicAdd(&s_buf_n, 1u)] = Entry{k1, k2};  // score >= ts: ties with the K-th kept
        }
    };

    // merge the buffer into the CTA's sorted list; publish the threshold and
    // the order statistics, then (warp 0) the threshold they certify
    auto merge = [&]() {
        cta_sort_desc(E, A.sort_n);
        for (uint32_t i = A.kpad + tid; i < A.sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
        if (tid == 0) {
            s_buf_n = 0;
            const Entry kth = E[A.keep - 1];
            if (kth.k1 != 0ull) {
                s_t1 = kth.k1;
                s_t2 = kth.k2;
                const unsigned int ok = static_cast<unsigned int>(kth.k1 >> 32);
                s_ts = okey_score(ok);
                atomicMax(&A.ctrl->gtau, ok);
            }
        }
        if (tid < kPruneMs && (1u << tid) <= A.keep) {
            const unsigned int ok = static_cast<unsigned int>(E[(1u << tid) - 1].k1 >> 32);
            if (ok != 0u) atomicMax(&A.pub[tid * gridDim.x + blockIdx.x], ok);
        }
        __syncthreads();
        if (tid < 32) {
            uint32_t best = 0;
            for (int mi = 0; mi < kPruneMs; ++mi) {
                const uint32_t jm = (A.keep + (1u << mi) - 1) >> mi;  // ceil(K / m)
                if ((1u << mi) > A.keep || jm > gridDim.x) continue;
                const volatile uint32_t *src = A.pub + mi * gridDim.x;
                for (uint32_t i = tid; i < gridDim.x; i += 32) sel[i] = src[i];
                __syncwarp();
                best = max(best, warp_kth_largest(sel, gridDim.x, jm));
                __syncwarp();
            }
            if (tid == 0 && best != 0u) atomicMax(&A.ctrl->gtau, best);
        }
    };

    for (;;) {
        __syncthreads();
        const unsigned int pn = min(s_pend_n, kPendCap);
        const int any = __syncthreads_or(valid || has_def);
        const int any_def = __syncthreads_or(has_def);
        // the queue is evaluated once it can employ every thread (or a thread
        // waits on it, or the work is done); a flush appends <= pn + 256 <= 768
        if (pn >= kThreads || any_def || (!any && pn > 0)) {
            if (s_buf_n + kPendCap + kThreads > A.buf_cap) merge();  // make room first
            unsigned long long t1 = s_t1, t2 = s_t2;
            float ts = s_ts;
            const unsigned int g = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->gtau);
            if ((static_cast<unsigned long long>(g) << 32) > t1) {
                t1 = static_cast<unsigned long long>(g) << 32;
                t2 = 0;
                ts = okey_score(g);
            }
            for (uint32_t i = tid; i < pn; i += kThreads) rescore(pend[i], t1, t2, ts);
            if (has_def) {
                rescore(def, t1, t2, ts);
                has_def = false;
            }
            __syncthreads();
            if (tid == 0) s_pend_n = 0;
            __syncthreads();
        }
        // merge when half full, and every kPruneMergeRounds rounds while the
        // buffer holds anything: the CTA's threshold and published keys then
        // follow the candidates it finds instead of waiting for a full buffer
        const unsigned int bn = s_buf_n;
        if (bn >= A.buf_cap / 2 || (bn > 0 && (!any || (round & (kPruneMergeRounds - 1)) == 0))) merge();
        if (!any) break;
        float ts = s_ts;
        const unsigned long long t1 = s_t1;
        if ((round++ & 7u) == 0) gk = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->gtau);
        if ((static_cast<unsigned long long>(gk) << 32) > t1) ts = okey_score(gk);
        const float tlo = __fsub_rd(ts, A.pc.err);
#pragma unroll 1
        for (int r = 0; r < kRounds && valid && !has_def; ++r) {
            const uint64_t s0 = seed_t + (p + 1) * kGolden;
            const PruneHead h = prune_head(A.sc, s0);
            const float b = prune_bound<kNb>(A, yt, s0, h.ea, h.eb);
            // immigrants are always scored; a NaN bound is never trusted
            if (h.imm || !(b < __fsub_rd(tlo, A.jb.c[h.jidx]))) {
                const unsigned int slot = atomicAdd(&s_pend_n, 1u);
                if (slot < kPendCap) {
                    pend[slot] = Pend{item, dcand, ddraw};
                } else {
                    has_def = true;
                    def = Pend{item, dcand, ddraw};
                }
            }
            p += h.len;
            ddraw += h.len;
            ++dcand;
            ++screened;
            if (--left == 0) {
                item = atomicAdd(&A.ctrl->next_item, 1u);
                valid = item < n_items;
                if (valid) {
                    const Item it = A.items[item];
                    seed_t = stream_seed(A.seed, it.stream);
                    p = it.draw0;
                    left = it.n;
                    dcand = 0;
                    ddraw = 0;
                    valid = left > 0;
                }
            }
        }
    }
    Entry *out = A.lists + static_cast<size_t>(blockIdx.x) * A.kpad;
    for (uint32_t i = tid; i < A.kpad; i += kThreads) out[i] = E[i];
    for (int o = 16; o > 0; o >>= 1) {
        screened += __shfl_down_sync(0xffffffffu, screened, o);
        exact += __shfl_down_sync(0xffffffffu, exact, o);
    }
    if ((tid & 31) == 0) {
        atomicAdd(&A.ctrl->screened, screened);
        atomicAdd(&A.ctrl->exact_evals, exact);
    }
}

// The crossover candidate's clamped parent genes y (first 16, in f32) and
// rt = sum_{k>=16} w_k y_k (kNb = 29), from its crossover bits.
template <int kNb>
__device__ __forceinline__ void prune_parents(const PruneArgs &A, const float *__restrict__ yt, uint64_t s0,
                                              uint32_t ea, uint32_t eb, float (&y)[16], float &rt) {
    constexpr int kYs = prune_stride<kNb>();
    const float *ya = yt + ea * kYs;
    const float *yb = yt + eb * kYs;
    uint64_t sb = s0 + 3 * kGolden;  // crossover bit draw of gene 0
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const uint32_t bw = draw_bitword(sb);
        sb += 2 * kGolden;
        y[k] = ((static_cast<int32_t>(bw) < 0) ? yb : ya)[k];
    }
    rt = 0.0f;
    if (kNb > 16) {
#pragma unroll
        for (int k = 16; k < kNb; ++k) {
            const uint32_t bw = draw_bitword(sb);
            sb += 2 * kGolden;
            rt = __fmaf_rn(A.m.wlin[k], ((static_cast<int32_t>(bw) < 0) ? yb : ya)[k], rt);
        }
    }
}

// The pruning screen with the bound's gradient on the tensor cores. Each
// 128-thread group runs rounds in step: every thread puts its candidate's
// parent genes (FP16) in row tid % 128 of the group's X tile (a zero row when
// it has no candidate), one thread issues tcgen05.mma (M 128, N 16, K 16,
// FP32 accumulation in TMEM), and each thread reads its row of Yh Qh back
// (tcgen05.ld). The rest is the FFMA form's: queue, merges, thresholds.
// A tensor-core wait that gives up stops the group's MMAs at once (tcp_round)
// and the CTA's screening at the next loop head; the error bit voids the
// result, and before TMEM is freed the issuer waits once more (bounded) for
// the MMA the wait gave up on.
// kFp16: the tile format of the bound's MMA (FP16, else BF16). kFp64: the
// precision form's ranking -- queued candidates are scored in FP64 and rank
// by that score rounded to f32 (the FP64 top-K; PruneConst::err covers the
// rounding of those scores too) -- instead of the reference's f32 order.
// The tensor-core screen's merge, out of line (its sort keeps its registers
// away from the screening loop's): the buffer into the CTA's sorted list, the
// CTA threshold and its published order statistics, then (warp 0) the
// threshold they certify. Every thread of the CTA calls it.
__device__ __noinline__ void prune_merge(const PruneArgs *A, Entry *E, uint32_t *sel, unsigned int *s_buf_n,
                                         unsigned long long *s_t1, unsigned long long *s_t2, float *s_ts) {
    const uint32_t tid = threadIdx.x;
    cta_sort_desc(E, A->sort_n);
    for (uint32_t i = A->kpad + tid; i < A->sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
    if (tid == 0) {
        *s_buf_n = 0;
        const Entry kth = E[A->keep - 1];
        if (kth.k1 != 0ull) {
            *s_t1 = kth.k1;
            *s_t2 = kth.k2;
            const unsigned int ok = static_cast<unsigned int>(kth.k1 >> 32);
            *s_ts = okey_score(ok);
            atomicMax(&A->ctrl->gtau, ok);
        }
    }
    if (tid < kPruneMs && (1u << tid) <= A->keep) {
        const unsigned int ok = static_cast<unsigned int>(E[(1u << tid) - 1].k1 >> 32);
        if (ok != 0u) atomicMax(&A->pub[tid * gridDim.x + blockIdx.x], ok);
    }
    __syncthreads();
    if (tid < 32) {
        uint32_t best = 0;
        for (int mi = 0; mi < kPruneMs; ++mi) {
            const uint32_t jm = (A->keep + (1u << mi) - 1) >> mi;
            if ((1u << mi) > A->keep || jm > gridDim.x) continue;
            const volatile uint32_t *src = A->pub + mi * gridDim.x;
            for (uint32_t i = tid; i < gridDim.x; i += 32) sel[i] = src[i];
            __syncwarp();
            best = max(best, warp_kth_largest(sel, gridDim.x, jm));
            __syncwarp();
        }
        if (tid == 0 && best != 0u) atomicMax(&A->ctrl->gtau, best);
    }
}

template <int kNb, bool kFp16, bool kFp64>
__global__ void __launch_bounds__(kThreads, 3) screen_pt_kernel(const __grid_constant__ PruneArgs A) {
    constexpr int kYs = prune_stride<kNb>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Entry *E = reinterpret_cast<Entry *>(smem_raw);
    // the elite table: only the queued candidates' full synthesis reads it;
    // in shared memory where that costs no CTA per SM, else through L1
    float *el_copy = reinterpret_cast<float *>(E + A.sort_n);
    const float *el = A.el_smem ? el_copy : A.el;
    Pend *pend = reinterpret_cast<Pend *>(el_copy + (A.el_smem ? (A.sc.ne + 1) * kNtot : 0u));
    float *yt = reinterpret_cast<float *>(pend + kPendCap);
    uint32_t *sel = reinterpret_cast<uint32_t *>(yt + A.sc.ne * kYs);
    __shared__ __align__(8) unsigned long long s_mbar[2];
    __shared__ uint32_t s_tbase;
    __shared__ unsigned int s_buf_n, s_pend_n;
    __shared__ uint32_t s_gbad[2], s_fail_phase[2];
    __shared__ unsigned long long s_t1, s_t2;
    __shared__ float s_ts;

    const uint32_t tid = threadIdx.x, warp = tid >> 5, grp = warp >> 2;
    const uint32_t base = smem_u32(smem_raw);
    const uint32_t after = smem_u32(sel + A.sel_cap);
    const uint32_t xs0 = (after + 1023u) & ~1023u;
    const uint32_t bts = xs0 + 2u * 4096u;
    for (uint32_t i = tid; i < A.sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
    if (A.el_smem)
        for (uint32_t i = tid; i < (A.sc.ne + 1) * kNtot; i += kThreads) el_copy[i] = A.el[i];
    for (uint32_t i = tid; i < A.sc.ne * kYs; i += kThreads) {
        const uint32_t r = i / kYs, k = i - r * kYs;
        yt[i] = (k < static_cast<uint32_t>(kNb)) ? fmaxf(fminf(A.el[r * kNtot + k], 1.0f), 0.0f) : 0.0f;
    }
    for (uint32_t i = tid; i < 128; i += kThreads)
        reinterpret_cast<uint32_t *>(smem_raw + (bts - base))[i] = reinterpret_cast<const uint32_t *>(A.tc.btile)[i];
    if (warp == 0) tc_alloc(smem_u32(&s_tbase), 32);
    if (tid == 0) {
        mbar_init(smem_u32(&s_mbar[0]), 1);
        mbar_init(smem_u32(&s_mbar[1]), 1);
        s_buf_n = 0;
        s_pend_n = 0;
        s_gbad[0] = s_gbad[1] = 0;
        s_fail_phase[0] = s_fail_phase[1] = 0;
        s_t1 = 0;
        s_t2 = 0;
        s_ts = -INFINITY;
    }
    const unsigned int n_items = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->n_items);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    TcGroup tg;
    tg.xs = xs0 + grp * 4096u;
    tg.mbar = smem_u32(&s_mbar[grp]);
    tg.tmem_d = s_tbase + 16u * grp;
    tg.tmem_ld = s_tbase + ((32u * (warp & 3u)) << 16) + 16u * grp;
    tg.adesc = tc_sdesc(tg.xs, 128, 256);
    tg.bdesc = tc_sdesc(bts, 128, 256);
    tg.idesc = tc_idesc(kFp16);
    tg.bar_id = 1u + grp;
    tg.phase = 0;
    tg.issuer = (tid & 127u) == 0;
    bool tc_ok = true;

    Entry *buf = E + A.kpad;
    uint32_t item = atomicAdd(&A.ctrl->next_item, 1u);
    bool valid = item < n_items;
    uint64_t seed_t = 0, p = 0;
    uint32_t left = 0, dcand = 0, ddraw = 0;
    if (valid) {
        const Item it = A.items[item];
        seed_t = stream_seed(A.seed, it.stream);
        p = it.draw0;
        left = it.n;
        valid = left > 0;
    }
    uint32_t screened = 0, exact = 0;  // per thread: far below 2^32
    unsigned int gk = 0;
    uint32_t round = 0;
    bool has_def = false;
    Pend def{0u, 0u, 0u};

    auto rescore = [&](const Pend &q, unsigned long long t1, unsigned long long t2, float ts) {
        const Item it = A.items[q.item];
        const float s = prune_rescore<kFp64>(&A, el, stream_seed(A.seed, it.stream), it.draw0 + q.ddraw,
                                             __fsub_rd(ts, A.err));
        ++exact;
        if (s >= ts) {
            const unsigned long long k1 =
                (static_cast<unsigned long long>(score_okey(s)) << 32) | static_cast<unsigned int>(~q.item);
            const unsigned long long k2 = (static_cast<unsigned long long>(~q.dcand) << 32) | q.ddraw;
            buf[atomicAdd(&s_buf_n, 1u)] = Entry{k1, k2};  // score >= ts: ties with the K-th kept
        }
    };

    auto merge = [&]() { prune_merge(&A, E, sel, &s_buf_n, &s_t1, &s_t2, &s_ts); };

    for (;;) {
        __syncthreads();
        const unsigned int pn = min(s_pend_n, kPendCap);
        // a group whose tensor-core wait gave up ends the CTA's screening
        const int stop = (s_gbad[0] | s_gbad[1]) != 0u;
        const int any = __syncthreads_or((valid || has_def) && !stop);
        const int any_def = __syncthreads_or(has_def);
        if (pn >= kThreads || any_def || (!any && pn > 0)) {
            if (s_buf_n + kPendCap + kThreads > A.buf_cap) merge();
            unsigned long long t1 = s_t1, t2 = s_t2;
            float ts = s_ts;
            const unsigned int g = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->gtau);
            if ((static_cast<unsigned long long>(g) << 32) > t1) {
                t1 = static_cast<unsigned long long>(g) << 32;
                t2 = 0;
                ts = okey_score(g);
            }
            for (uint32_t i = tid; i < pn; i += kThreads) rescore(pend[i], t1, t2, ts);
            if (has_def) {
                rescore(def, t1, t2, ts);
                has_def = false;
            }
            __syncthreads();
            if (tid == 0) s_pend_n = 0;
            __syncthreads();
        }
        const unsigned int bn = s_buf_n;
        if (bn >= A.buf_cap / 2 || (bn > 0 && (!any || (round & (kPruneMergeRounds - 1)) == 0))) merge();
        if (!any) break;
        float ts = s_ts;
        const unsigned long long t1 = s_t1;
        if ((round++ & 7u) == 0) gk = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->gtau);
        if ((static_cast<unsigned long long>(gk) << 32) > t1) ts = okey_score(gk);
        const float tlo = __fsub_rd(ts, A.tc.err);
#pragma unroll 1
        for (int r = 0; r < kRounds; ++r) {
            const bool act = valid && !has_def;
            uint32_t pk[8];
            float rt = 0.0f;
            PruneHead h{0u, 0u, kNoJump, 0u, false};
            if (act) {
                const uint64_t s0 = seed_t + (p + 1) * kGolden;
                h = prune_head(A.sc, s0);
                float y[16];
                prune_parents<kNb>(A, yt, s0, h.ea, h.eb, y, rt);
#pragma unroll
                for (int j = 0; j < 8; ++j) pk[j] = pack2(y[2 * j], y[2 * j + 1], kFp16);
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j) pk[j] = 0u;
            }
            float d[16];
            if (!tcp_round(tg, pk, tid & 127u, d, &s_gbad[grp], &s_fail_phase[grp])) tc_ok = false;
            if (act) {
                float f2 = 0.0f, l1 = 0.0f;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const float2 yh = kFp16 ? __half22float2(*reinterpret_cast<const __half2 *>(&pk[j]))
                                            : __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&pk[j]));
                    const float g0 = __fmaf_rn(d[2 * j], A.tc.dscale, A.m.wlin[2 * j]);
                    const float g1 = __fmaf_rn(d[2 * j + 1], A.tc.dscale, A.m.wlin[2 * j + 1]);
                    l1 = __fadd_rn(__fadd_rn(l1, fabsf(g0)), fabsf(g1));
                    f2 = __fmaf_rn(yh.x, __fadd_rn(g0, A.m.wlin[2 * j]), f2);
                    f2 = __fmaf_rn(yh.y, __fadd_rn(g1, A.m.wlin[2 * j + 1]), f2);
                }
                const float b = __fadd_rn(__fmaf_rn(A.tc.s, l1, __fmaf_rn(0.5f, f2, __fadd_rn(A.m.w16, rt))),
                                          A.tc.c0);
                if (h.imm || !(b < __fsub_rd(tlo, A.jb.c[h.jidx]))) {
                    const unsigned int slot = atomicAdd(&s_pend_n, 1u);
                    if (slot < kPendCap) {
                        pend[slot] = Pend{item, dcand, ddraw};
                    } else {
                        has_def = true;
                        def = Pend{item, dcand, ddraw};
                    }
                }
                p += h.len;
                ddraw += h.len;
                ++dcand;
                ++screened;
                if (--left == 0) {
                    item = atomicAdd(&A.ctrl->next_item, 1u);
                    valid = item < n_items;
                    if (valid) {
                        const Item it = A.items[item];
                        seed_t = stream_seed(A.seed, it.stream);
                        p = it.draw0;
                        left = it.n;
                        dcand = 0;
                        ddraw = 0;
                        valid = left > 0;
                    }
                }
            }
        }
    }
    Entry *out = A.lists + static_cast<size_t>(blockIdx.x) * A.kpad;
    for (uint32_t i = tid; i < A.kpad; i += kThreads) out[i] = E[i];
    unsigned long long scr = screened, exa = exact;
    for (int o = 16; o > 0; o >>= 1) {
        scr += __shfl_down_sync(0xffffffffu, scr, o);
        exa += __shfl_down_sync(0xffffffffu, exa, o);
    }
    if ((tid & 31) == 0) {
        atomicAdd(&A.ctrl->screened, scr);
        atomicAdd(&A.ctrl->exact_evals, exa);
    }
    if (!tc_ok) atomicOr(&A.ctrl->err, kErrTc);
    __syncthreads();
    if (s_gbad[grp] != 0u && tg.issuer) (void)mbar_wait(tg.mbar, s_fail_phase[grp]);  // bounded
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tc_dealloc(s_tbase, 32);
}

using PruneScreenFn = void (*)(PruneArgs);

// The pruning kernel of a plan: FFMA or tensor-core bound; for the latter
// the tile format and the ranking (f32 reference order, or FP64 for the
// precision form, whose BF16 flag takes BF16 tiles).
PruneScreenFn screen_p_fn(int nb, bool tc, bool fp16, bool fp64) {
    const bool t = nb > 16;
    if (!tc) return t ? screen_p_kernel<kNtot> : screen_p_kernel<16>;
    if (!fp64) return t ? screen_pt_kernel<kNtot, true, false> : screen_pt_kernel<16, true, false>;
    if (fp16) return t ? screen_pt_kernel<kNtot, true, true> : screen_pt_kernel<16, true, true>;
    return t ? screen_pt_kernel<kNtot, false, true> : screen_pt_kernel<16, false, true>;
}

// Shared memory of the pruning screen: the sort buffer, the queue, the
// clamped parent table and the selection scratch of the published keys (one
// per CTA, at most 8 CTAs per SM), with el_smem the elite table; the
// tensor-core form adds its two X tiles and B tile (1 KB aligned).
size_t prune_smem(uint32_t sort_n, int ne, int nb, int num_sms, bool tc, bool el_smem) {
    const size_t ys = nb > 16 ? kNtot : 17;
    const size_t n = static_cast<size_t>(sort_n) * sizeof(Entry) + kPendCap * sizeof(Pend) +
                     static_cast<size_t>(ne) * ys * sizeof(float) + 8ull * num_sms * sizeof(uint32_t) +
                     (el_smem ? static_cast<size_t>(ne + 1) * kNtot * sizeof(float) : 0);
    return tc ? n + 1024 + 2 * 4096 + 512 : n;
}

// The bound's constants for a model whose filter bound is finite and a
// mutation width the fast delta form handles. *nb: crossover genes the bound
// draws (16 when every linear weight past gene 15 is zero). Returns false
// when the bound cannot be certified (non-finite sums).
bool make_prune(const csx_model &m, float sigma, PruneConst *pc, int *nb) {
    const double s = std::min(std::fabs(static_cast<double>(sigma)) + std::ldexp(1.0, -24), 1.0);
    double qsum = 0.0, qpos = 0.0, lsum = 0.0, tail = 0.0;
    bool tail_nz = false;
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) {
            const double q = static_cast<double>(m.w_quad[i * 16 + j]);
            qsum += std::fabs(q);
            qpos += (i == j) ? std::max(q, 0.0) : std::fabs(q);
        }
    for (int k = 0; k < kNtot; ++k) {
        const double w = static_cast<double>(m.w_lin[k]);
        lsum += std::fabs(w);
        if (k >= 16) {
            tail += std::fabs(w);
            tail_nz = tail_nz || w != 0.0;
        }
    }
    for (int j = 0; j < 16; ++j)
        for (int k = 0; k < 16; ++k) {
            const float q = j >= k ? m.w_quad[j * 16 + k] : m.w_quad[k * 16 + j];
            pc->qs[j][k] = (j == k) ? 2.0f * q : q;  // exact: the weights are finite and below 1e30
        }
    const double up = 1.0 + std::ldexp(1.0, -20);
    const double c0 = (s * tail + s * s * qpos) * up;
    const double u = std::ldexp(1.0, -24);
    auto gamma = [u](double n) { return n * u / (1.0 - n * u); };
    const double w16 = 16.0 * std::fabs(static_cast<double>(m.w0));
    const double a_bound = w16 + 3.0 * lsum + 4.0 * qsum + c0;  // magnitudes the bound's f32 sums reach
    const double a_ref = w16 + lsum + qsum;                      // the reference order's (genes in [0, 1])
    const double err = (2.0 * gamma(64) * a_bound + gamma(35) * a_ref) * up + 1e-30;
    if (!std::isfinite(c0) || !std::isfinite(err) || err > 1e30) return false;
    pc->s = std::nextafter(static_cast<float>(s), INFINITY);
    pc->c0 = c0 > 0.0 ? std::nextafter(static_cast<float>(c0), INFINITY) : 0.0f;
    pc->err = std::nextafter(static_cast<float>(err), INFINITY);
    *nb = tail_nz ? kNtot : 16;
    return true;
}

// The tensor-core form's tile, box and error share for a model whose
// PruneConst is set. The bound is centred on yh = fp16(y) (or bf16(y)) in
// [0, 1], |yh - y| <= u = 2^-12 (2^-9 for BF16), so each gene lies within
// s' = s + u of it; c0 takes s'. Qs * 2^-e is rounded to the tile format (e:
// the largest entry lands in [2^14, 2^15)); with the MMA's exact products
// and an FP32 accumulation taken as losing at most 2^-18 of its absolute sum,
//   |2^e D_k - (Qs yh)_k| <= eps_k = sum_j (dq_kj + 2^-18 (|Qs_kj| + dq_kj)),
// dq_kj = |2^e round(Qs_kj 2^-e) - Qs_kj| (computed exactly here). The bound
// uses grad_k = wl_k + 2^e D_k in s' sum |grad_k| and in f(yh) = 16 w0 +
// sum_k yh_k (grad_k + wl_k) / 2, so it rises by at most (s' + 1/2) sum_k
// eps_k over the exact-gradient bound at yh.
bool make_prune_tc(const csx_model &m, const PruneConst &pc, bool fp16, PruneTc *t) {
    double qs[16][16], qmax = 0.0;
    for (int n = 0; n < 16; ++n)
        for (int k = 0; k < 16; ++k) {
            qs[n][k] = static_cast<double>(pc.qs[n][k]);
            qmax = std::max(qmax, std::fabs(qs[n][k]));
        }
    int e = 0;
    if (qmax > 0.0) {
        e = std::ilogb(qmax) + 1 - 15;  // qmax * 2^-e in [2^14, 2^15)
        if (e < -126 || e > 127) return false;
    }
    double eps = 0.0;
    std::memset(t->btile, 0, sizeof(t->btile));
    for (int n = 0; n < 16; ++n)
        for (int k = 0; k < 16; ++k) {
            const float x = static_cast<float>(std::ldexp(qs[n][k], -e));  // exact: a power-of-two scaling
            uint16_t bits;
            double back;
            if (fp16) {
                const __half h = __float2half_rn(x);
                bits = *reinterpret_cast<const uint16_t *>(&h);
                back = std::ldexp(static_cast<double>(__half2float(h)), e);
            } else {
                const __nv_bfloat16 h = __float2bfloat16_rn(x);
                bits = *reinterpret_cast<const uint16_t *>(&h);
                back = std::ldexp(static_cast<double>(__bfloat162float(h)), e);
            }
            if (!std::isfinite(back)) return false;
            const double dq = std::fabs(back - qs[n][k]);
            eps += dq + std::ldexp(1.0, -18) * (std::fabs(qs[n][k]) + dq);
            const int off = (n >> 3) * 256 + (k >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2;
            t->btile[off / 2] = bits;
        }
    const double up = 1.0 + std::ldexp(1.0, -20);
    const double s = std::min(static_cast<double>(pc.s) + std::ldexp(1.0, fp16 ? -12 : -9), 1.0);
    double qpos = 0.0, tail = 0.0;
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) {
            const double q = static_cast<double>(m.w_quad[i * 16 + j]);
            qpos += (i == j) ? std::max(q, 0.0) : std::fabs(q);
        }
    for (int k = 16; k < kNtot; ++k) tail += std::fabs(static_cast<double>(m.w_lin[k]));
    const double c0 = (s * tail + s * s * qpos) * up;
    const double err = (static_cast<double>(pc.err) + (s + 0.5) * eps) * up;
    if (!std::isfinite(err) || err > 1e30 || !std::isfinite(c0)) return false;
    t->dscale = std::ldexp(1.0f, e);
    t->s = std::nextafter(static_cast<float>(s), INFINITY);
    t->c0 = c0 > 0.0 ? std::nextafter(static_cast<float>(c0), INFINITY) : 0.0f;
    t->err = std::nextafter(static_cast<float>(err), INFINITY);
    return true;
}

}  // namespace csx

namespace csx {

// CTAs per SM of a pruning screen with this shared memory (228 KB per SM, 1 KB
// reserved per CTA; at most 3, the register limit of the tensor-core form).
inline int prune_fit(size_t smem) { return std::min(3, static_cast<int>((228u << 10) / (smem + 1024))); }

// Whether the elite table goes to shared memory: where it costs no CTA per SM
// (the queue's synthesis reads it; through L1 it measured 0.7% slower at 64
// elites, and at 256 elites the table would hold the screen to two CTAs per SM).
inline bool prune_el_smem(uint32_t sort_n, int ne, int nb, int num_sms, bool tc, size_t max_smem) {
    const size_t with = prune_smem(sort_n, ne, nb, num_sms, tc, true);
    return with + 1024 <= max_smem &&
           prune_fit(with) >= prune_fit(prune_smem(sort_n, ne, nb, num_sms, tc, false));
}

}  // namespace csx
