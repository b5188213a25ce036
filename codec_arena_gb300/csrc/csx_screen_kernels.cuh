// csx_screen_kernels.cuh — the screen kernels (exact form, filter form with
// its queued exact order, precision form on the tensor cores), the merge
// tree and survivor regeneration.
// Part of csx_screen.cu's translation unit (included there, in order); not a
// standalone header.
#pragma once

namespace csx {

// ---- 4. screen ----------------------------------------------------------------

struct ScreenArgs {
    DevModel m;
    SynthConst sc;
    uint64_t seed;
    const float *el;  // (ne + 1) x 29
    const Item *items;
    Ctrl *ctrl;
    Entry *lists;     // gridDim.x x kpad
    uint32_t keep, kpad, sort_n, buf_cap;
    float err;        // bound on |filter score - exact score| (filter mode)
    JumpBound jb;     // added to err for a candidate with a jump (filter mode)
};

// The screen on the full quadratic surface: the same pipeline, the
// candidates scored by synth_full (no filter: its FMA order is the defined
// score).
struct FullScreenArgs : ScreenArgs {
    FullModel fm;
};

// The score of the candidate at p (header h) under the call's surface.
template <bool kFastDelta>
__device__ __forceinline__ float cand_score(const ScreenArgs &A, const float *el, uint64_t seed_t, uint64_t p,
                                            const CandHead &h) {
    return synth_score<kFastDelta, false>(A.m, A.sc, el, seed_t, p, h, nullptr);
}
template <bool kFastDelta>
__device__ __forceinline__ float cand_score(const FullScreenArgs &A, const float *el, uint64_t seed_t,
                                            uint64_t p, const CandHead &h) {
    return synth_full<kFastDelta, false>(A.fm, A.sc, el, seed_t, p, h, nullptr);
}

// The same with the genes kept (regeneration of survivors).
template <bool kFastDelta>
__device__ __forceinline__ float cand_genes(const DevModel &m, const SynthConst &sc, const float *el,
                                            uint64_t seed_t, uint64_t p, const CandHead &h, float *genes) {
    return synth_score<kFastDelta, true>(m, sc, el, seed_t, p, h, genes);
}
template <bool kFastDelta>
__device__ __forceinline__ float cand_genes(const FullModel &m, const SynthConst &sc, const float *el,
                                            uint64_t seed_t, uint64_t p, const CandHead &h, float *genes) {
    return synth_full<kFastDelta, true>(m, sc, el, seed_t, p, h, genes);
}

// Bitonic sort of E[0..n) (n a power of two), best entry first.
__device__ void cta_sort_desc(Entry *E, uint32_t n) {
    for (uint32_t size = 2; size <= n; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = threadIdx.x; i < (n >> 1); i += blockDim.x) {
                const uint32_t lo = 2 * i - (i & (stride - 1));
                const uint32_t hi = lo + stride;
                const bool desc = (lo & size) == 0;
                const Entry a = E[lo], b = E[hi];
                if (desc ? better(b, a) : better(a, b)) {
                    E[lo] = b;
                    E[hi] = a;
                }
            }
            __syncthreads();
        }
    }
}

// The reference-order score of one candidate, out of line: it runs only for
// candidates the filter cannot rule out, and keeping it out of the caller
// stops the compiler from holding both evaluations' values live at once.
template <bool kFastDelta>
__device__ __noinline__ float exact_score_at(const ScreenArgs *__restrict__ A, const float *el,
                                             uint64_t seed_t, uint64_t p) {
    const CandHead h = cand_head(A->sc, seed_t, p);
    return synth_score<kFastDelta, false, true>(A->m, A->sc, el, seed_t, p, h, nullptr);
}

// The exact form (CSX_FLAG_EXACT_ALL, or a model whose filter bound is not
// finite): every candidate scored in the reference's f32 order. With
// FullScreenArgs, every candidate scored on the full surface.
template <bool kFastDelta, class Args = ScreenArgs>
__global__ void __launch_bounds__(kThreads, 3) screen_kernel(const __grid_constant__ Args A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Entry *E = reinterpret_cast<Entry *>(smem_raw);
    float *el = reinterpret_cast<float *>(E + A.sort_n);
    __shared__ unsigned int s_buf_n;
    __shared__ unsigned long long s_t1, s_t2;
    __shared__ float s_ts;

    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i < A.sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
    for (uint32_t i = tid; i < (A.sc.ne + 1) * kNtot; i += kThreads) el[i] = A.el[i];
    if (tid == 0) {
        s_buf_n = 0;
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
    unsigned long long screened = 0;
    unsigned int gk = 0;
    uint32_t round = 0;
    // An append that finds the buffer full is held here and the thread pauses
    // until the next merge (which the full buffer forces), so no entry is lost
    // and the buffer never needs room for a whole round of appends.
    bool has_def = false;
    Entry def{0ull, 0ull};

    for (;;) {
        __syncthreads();
        const unsigned int bn = s_buf_n;  // nobody appends until after the next barrier
        const int any = __syncthreads_or(valid || has_def);
        if (bn >= A.buf_cap / 2 || (!any && bn > 0)) {
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
            __syncthreads();
        }
        if (!any) break;
        if (has_def) {  // the merge above emptied the buffer: room for every held entry
            const unsigned int slot = atomicAdd(&s_buf_n, 1u);
            buf[slot] = def;
            has_def = false;
        }
        unsigned long long t1 = s_t1, t2 = s_t2;
        float ts = s_ts;
        if ((round++ & 7u) == 0) gk = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->gtau);
        if ((static_cast<unsigned long long>(gk) << 32) > t1) {
            t1 = static_cast<unsigned long long>(gk) << 32;
            t2 = 0;
            ts = okey_score(gk);
        }
#pragma unroll 1
        for (int r = 0; r < kRounds && valid && !has_def; ++r) {
            const CandHead h = cand_head(A.sc, seed_t, p);
            const float s = cand_score<kFastDelta>(A, el, seed_t, p, h);
            // every candidate scoring at least the threshold enters the buffer,
            // ties with the running K-th score included: the final list's
            // (K+1)-th entry is then exact (exact-tie detection)
            if (s >= ts) {
                const unsigned long long k1 =
                    (static_cast<unsigned long long>(score_okey(s)) << 32) | static_cast<unsigned int>(~item);
                const unsigned long long k2 =
                    (static_cast<unsigned long long>(~dcand) << 32) | ddraw;
                const unsigned int slot = atomicAdd(&s_buf_n, 1u);
                if (slot < A.buf_cap) {
                    buf[slot] = Entry{k1, k2};
                } else {
                    has_def = true;
                    def = Entry{k1, k2};
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
    // CTA list out (the last iteration merged any pending buffer)
    Entry *out = A.lists + static_cast<size_t>(blockIdx.x) * A.kpad;
    for (uint32_t i = tid; i < A.kpad; i += kThreads) out[i] = E[i];
    // screened count: warp reduce then one atomic per warp
    for (int o = 16; o > 0; o >>= 1) screened += __shfl_down_sync(0xffffffffu, screened, o);
    if ((tid & 31) == 0) atomicAdd(&A.ctrl->screened, screened);
}

// The filter form with the reference-order evaluation deferred: a candidate
// whose filter score is within the bound of the threshold goes to a shared
// queue, and at the next merge all threads evaluate the queue in the
// reference's f32 order -- whole warps, instead of one lane evaluating while
// the other 31 of its warp wait. The buffer fills only from the queue, and
// every fill is sorted at once, so it always has room (queue + one held entry
// per thread <= 768 <= sort_n - kpad).
// Two CTAs per SM with up to 128 registers: 1% faster than three at 80
// (measured; the other screen kernels are faster at three).
template <bool kFastDelta>
__global__ void __launch_bounds__(kThreads, 2) screen_q_kernel(const __grid_constant__ ScreenArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Entry *E = reinterpret_cast<Entry *>(smem_raw);
    float *el = reinterpret_cast<float *>(E + A.sort_n);
    Pend *pend = reinterpret_cast<Pend *>(el + (A.sc.ne + 1) * kNtot);
    __shared__ unsigned int s_buf_n, s_pend_n;
    __shared__ unsigned long long s_t1, s_t2;
    __shared__ float s_ts;

    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i < A.sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
    for (uint32_t i = tid; i < (A.sc.ne + 1) * kNtot; i += kThreads) el[i] = A.el[i];
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
        const float s = exact_score_at<kFastDelta>(&A, el, stream_seed(A.seed, it.stream), it.draw0 + q.ddraw);
        ++exact;
        if (s >= ts) {
            const unsigned long long k1 =
                (static_cast<unsigned long long>(score_okey(s)) << 32) | static_cast<unsigned int>(~q.item);
            const unsigned long long k2 = (static_cast<unsigned long long>(~q.dcand) << 32) | q.ddraw;
            buf[atomicAdd(&s_buf_n, 1u)] = Entry{k1, k2};  // score >= ts: ties with the K-th kept
        }
    };

    // merge the buffer into the CTA's sorted list; publishes the threshold
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
        __syncthreads();
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
        const unsigned int bn = s_buf_n;
        if (bn >= A.buf_cap / 2 || (!any && bn > 0)) merge();
        if (!any) break;
        float ts = s_ts;
        const unsigned long long t1 = s_t1;
        if ((round++ & 7u) == 0) gk = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->gtau);
        if ((static_cast<unsigned long long>(gk) << 32) > t1) ts = okey_score(gk);
        const float tlo = __fsub_rd(ts, A.err);
#pragma unroll 1
        for (int r = 0; r < kRounds && valid && !has_def; ++r) {
            const CandHead h = cand_head(A.sc, seed_t, p);
            const float s = synth_score<kFastDelta, false, false>(A.m, A.sc, el, seed_t, p, h, nullptr);
            if (s >= __fsub_rd(tlo, A.jb.c[h.jidx])) {
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

// ---- 5. merge tree ------------------------------------------------------------------

// Merge lists 2j and 2j+1 of `in` (nl lists of kpad entries, best first) into
// list j of `out`; S holds 2 * kpad entries of shared memory.
__device__ void merge_pair(const Entry *__restrict__ in, uint32_t nl, Entry *__restrict__ out, uint32_t kpad,
                           uint32_t j, Entry *S) {
    const uint32_t a = 2 * j, b = 2 * j + 1;
    const Entry *la = in + static_cast<size_t>(a) * kpad;
    Entry *o = out + static_cast<size_t>(j) * kpad;
    if (b >= nl) {
        for (uint32_t i = threadIdx.x; i < kpad; i += blockDim.x) o[i] = la[i];
        return;
    }
    const Entry *lb = in + static_cast<size_t>(b) * kpad;
    for (uint32_t i = threadIdx.x; i < kpad; i += blockDim.x) {
        S[i] = la[i];
        S[2 * kpad - 1 - i] = lb[i];  // descending ++ ascending: bitonic
    }
    __syncthreads();
    for (uint32_t stride = kpad; stride > 0; stride >>= 1) {
        for (uint32_t i = threadIdx.x; i < kpad; i += blockDim.x) {
            const uint32_t lo = 2 * i - (i & (stride - 1));
            const uint32_t hi = lo + stride;
            const Entry x = S[lo], y = S[hi];
            if (better(y, x)) {
                S[lo] = y;
                S[hi] = x;
            }
        }
        __syncthreads();
    }
    for (uint32_t i = threadIdx.x; i < kpad; i += blockDim.x) o[i] = S[i];
}

__global__ void merge_kernel(const Entry *__restrict__ in, uint32_t nl, Entry *__restrict__ out,
                             uint32_t kpad) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    merge_pair(in, nl, out, kpad, blockIdx.x, reinterpret_cast<Entry *>(smem_raw));
}

// ---- 6. regenerate survivors ------------------------------------------------------

// Survivor q of a final list: regenerate its genes and lineage from its
// (item, candidate, draw) key and check the score bits against the key.
template <bool kFastDelta, class Model>
__device__ void regen_one(const Model &m, const SynthConst &sc, uint64_t seed, const float *el,
                          const Item *items, Ctrl *ctrl, const Entry *fin, uint32_t keep,
                          const unsigned long long *ids, const unsigned int *tribes, csx_survivor *out,
                          uint32_t q) {
    if (q >= keep) return;
    const Entry e = fin[q];
    const bool real = e.k1 != 0ull;
    const bool next_real = (q + 1 < keep) ? (fin[q + 1].k1 != 0ull) : false;
    if (q == 0 && !real) ctrl->n_out = 0;
    if (real && !next_real) ctrl->n_out = q + 1;
    if (!real) return;
    const uint32_t item = ~static_cast<uint32_t>(e.k1);
    const uint32_t dcand = ~static_cast<uint32_t>(e.k2 >> 32);
    const uint32_t ddraw = static_cast<uint32_t>(e.k2);
    const Item it = items[item];
    const uint64_t seed_t = stream_seed(seed, it.stream);
    const uint64_t draw = it.draw0 + ddraw;
    const CandHead h = cand_head(sc, seed_t, draw);
    float genes[kNtot];
    const float s = cand_genes<kFastDelta>(m, sc, el, seed_t, draw, h, genes);
    if (score_okey(s) != static_cast<unsigned int>(e.k1 >> 32)) atomicOr(&ctrl->err, kErrRegen);
    csx_survivor v;
    v.score = s;
    v.tribe = tribes[h.ea];
    v.pa = ids[h.ea];
    v.pb = ids[h.eb];
    v.stream = it.stream;
    v.index = it.idx0 + dcand;
    v.draw = draw;
#pragma unroll
    for (int k = 0; k < kNtot; ++k) v.g[k] = genes[k];
    v.reserved = 0;
    out[q] = v;
}

template <bool kFastDelta>
__global__ void regen_kernel(const __grid_constant__ ScreenArgs A, const Entry *__restrict__ fin,
                             const unsigned long long *__restrict__ ids,
                             const unsigned int *__restrict__ tribes, csx_survivor *__restrict__ out,
                             unsigned long long *__restrict__ result) {
    (void)result;
    regen_one<kFastDelta>(A.m, A.sc, A.seed, A.el, A.items, A.ctrl, fin, A.keep, ids, tribes, out,
                          blockIdx.x * blockDim.x + threadIdx.x);
}

template <bool kFastDelta>
__global__ void regen_full_kernel(const __grid_constant__ FullScreenArgs A, const Entry *__restrict__ fin,
                                  const unsigned long long *__restrict__ ids,
                                  const unsigned int *__restrict__ tribes, csx_survivor *__restrict__ out) {
    regen_one<kFastDelta>(A.fm, A.sc, A.seed, A.el, A.items, A.ctrl, fin, A.keep, ids, tribes, out,
                          blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void result_kernel(const Ctrl *__restrict__ ctrl, unsigned long long *__restrict__ result) {
    if (threadIdx.x == 0) {
        result[0] = ctrl->n_out;
        result[1] = ctrl->screened;
        result[2] = ctrl->err;
        result[3] = ctrl->n_items - ctrl->item_begin;
    }
}

// ---- precision form (tensor cores), used by make_plan / enqueue_screen -------------

int make_tc_model(const csx_model &m, bool fp16, TcModel *t);

constexpr float kTcBand = 1e-3f;  // relative band below the K-th score rescored in FP64
constexpr int kTcCtasPerSm = 3;   // precision-form screen CTAs per SM
constexpr size_t kTcSmemExtra = 512 * 12 + 1024 + 2 * 4096 + 512;  // band queue, alignment slack, two X tiles, B tile

struct TcScreenArgs {
    ScreenArgs A;
    TcModel tm;
    float band;     // relative band below the threshold
    float err_abs;  // certified bound on |tensor-core score - exact score|: the band is never narrower
};

int tc_error_bound(const csx_model &m, bool fp16, float *out);

__device__ __forceinline__ double score64_genes(const DevModel &m, const float (&g)[kNtot]) {
    double s = 16.0 * static_cast<double>(m.w0);
#pragma unroll
    for (int k = 0; k < kNtot; ++k) s = fma(static_cast<double>(m.wlin[k]), static_cast<double>(g[k]), s);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        double t = 0.0;
#pragma unroll
        for (int j = 0; j <= i; ++j) t = fma(static_cast<double>(m.wq[tri(i, j)]), static_cast<double>(g[j]), t);
        s = fma(t, static_cast<double>(g[i]), s);
    }
    return s;
}

// FP64 score of the candidate at p (genes regenerated exactly), out of line.
template <bool kFastDelta>
__device__ __noinline__ double score64_at(const DevModel *m, const SynthConst *sc, const float *el, uint64_t seed_t,
                                          uint64_t p) {
    const CandHead h = cand_head(*sc, seed_t, p);
    float g[kNtot];
#pragma unroll
    for (int k = 16; k < kNtot; ++k) g[k] = 0.0f;  // left so without a tail: weight +-0 times 0
    (void)synth_score<kFastDelta, true, true, DevModel, true, true>(*m, *sc, el, seed_t, p, h, g);
    return score64_genes(*m, g);
}

// The screen in the precision form: the quadratic block of every candidate on
// the tensor cores (two 128-thread groups, one MMA per group per round).
// Candidates whose tensor-core score is within the band of the CTA threshold
// go to a shared queue; at the next merge all threads score the queue in FP64
// (whole warps, not one lane per warp) and the results enter the top-K, ranked
// by the FP64 score rounded to f32. Rounds are group-uniform: a thread without
// work feeds a zero row.
template <bool kFastDelta, bool kFp16>
__global__ void __launch_bounds__(kThreads, 3) screen_tc_kernel(const __grid_constant__ TcScreenArgs P) {
    const ScreenArgs &A = P.A;
    extern __shared__ __align__(16) unsigned char smem_raw[];  // tiles are aligned by address below
    Entry *E = reinterpret_cast<Entry *>(smem_raw);
    float *el = reinterpret_cast<float *>(E + A.sort_n);
    Pend *pend = reinterpret_cast<Pend *>(el + (A.sc.ne + 1) * kNtot);
    __shared__ __align__(8) unsigned long long s_mbar[2];
    __shared__ uint32_t s_tbase;
    __shared__ uint32_t s_gbad[2], s_fail_phase[2];
    __shared__ unsigned int s_buf_n, s_pend_n;
    __shared__ unsigned long long s_t1, s_t2;
    __shared__ float s_ts;

    const uint32_t tid = threadIdx.x, warp = tid >> 5, grp = warp >> 2;
    const uint32_t base = smem_u32(smem_raw);
    const uint32_t after = smem_u32(pend + kPendCap);
    const uint32_t xs0 = (after + 1023u) & ~1023u;
    const uint32_t bts = xs0 + 2u * 4096u;
    for (uint32_t i = tid; i < A.sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
    for (uint32_t i = tid; i < (A.sc.ne + 1) * kNtot; i += kThreads) el[i] = A.el[i];
    for (uint32_t i = tid; i < 128; i += kThreads)
        reinterpret_cast<uint32_t *>(smem_raw + (bts - base))[i] = reinterpret_cast<const uint32_t *>(P.tm.btile)[i];
    if (warp == 0) tc_alloc(smem_u32(&s_tbase), 32);
    if (tid == 0) {
        mbar_init(smem_u32(&s_mbar[0]), 1);
        mbar_init(smem_u32(&s_mbar[1]), 1);
        s_gbad[0] = s_gbad[1] = 0;
        s_fail_phase[0] = s_fail_phase[1] = 0;
        s_buf_n = 0;
        s_pend_n = 0;
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
    unsigned long long screened = 0, exact = 0;
    unsigned int gk = 0;
    uint32_t round = 0;
    bool has_def = false;  // holds a band candidate the full queue could not take
    Pend def{0u, 0u, 0u};

    // FP64 score of a queued candidate; enters the buffer if it beats the threshold.
    auto rescore = [&](const Pend &q, unsigned long long t1, unsigned long long t2, float ts) {
        const Item it = A.items[q.item];
        const uint64_t st = stream_seed(A.seed, it.stream);
        const float sf = static_cast<float>(score64_at<kFastDelta>(&A.m, &A.sc, el, st, it.draw0 + q.ddraw));
        ++exact;
        if (sf >= ts) {
            const unsigned long long k1 =
                (static_cast<unsigned long long>(score_okey(sf)) << 32) | static_cast<unsigned int>(~q.item);
            const unsigned long long k2 = (static_cast<unsigned long long>(~q.dcand) << 32) | q.ddraw;
            buf[atomicAdd(&s_buf_n, 1u)] = Entry{k1, k2};  // score >= ts: ties with the K-th kept
        }
    };

    // merge the buffer into the CTA's sorted list; publishes the threshold
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
        __syncthreads();
    };

    for (;;) {
        __syncthreads();
        const unsigned int pn = min(s_pend_n, kPendCap);
        // a group whose tensor-core wait gave up ends the CTA's screening
        const int stop = (s_gbad[0] | s_gbad[1]) != 0u;
        const int any = __syncthreads_or((valid || has_def) && !stop);
        const int any_def = __syncthreads_or(has_def);
        // the queue is scored once it can employ every thread (or a thread
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
        const unsigned int bn = s_buf_n;
        if (bn >= A.buf_cap / 2 || (!any && bn > 0)) merge();
        if (!any) break;
        unsigned long long t1 = s_t1;
        float ts = s_ts;
        if ((round++ & 7u) == 0) gk = *reinterpret_cast<volatile unsigned int *>(&A.ctrl->gtau);
        if ((static_cast<unsigned long long>(gk) << 32) > t1) {
            t1 = static_cast<unsigned long long>(gk) << 32;
            ts = okey_score(gk);
        }
        const float tlo = __fsub_rd(ts, fmaxf(__fmul_ru(P.band, fabsf(ts)), P.err_abs));
#pragma unroll 1
        for (int r = 0; r < kRounds; ++r) {
            const bool act = valid && !has_def;
            float R = 0.0f, x[16];
            uint32_t pk[8];
            uint32_t len = 0;
            float jb = 0.0f;
            if (act) {
                const CandHead h = cand_head(A.sc, seed_t, p);
                synth_tc<kFastDelta, kFp16>(P.tm, A.sc, el, seed_t, p, h, R, x, pk);
                len = h.len;
                jb = A.jb.c[h.jidx];
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j) pk[j] = 0u;
#pragma unroll
                for (int i = 0; i < 16; ++i) x[i] = 0.0f;
            }
            float y[16];
            if (!tcp_round(tg, pk, tid & 127u, y, &s_gbad[grp], &s_fail_phase[grp])) tc_ok = false;
            if (act) {
                float s = R;
#pragma unroll
                for (int i = 0; i < 16; ++i) s = __fmaf_rn(x[i], y[i], s);
                if (s >= __fsub_rd(tlo, jb)) {
                    const unsigned int slot = atomicAdd(&s_pend_n, 1u);
                    if (slot < kPendCap) {
                        pend[slot] = Pend{item, dcand, ddraw};
                    } else {
                        has_def = true;
                        def = Pend{item, dcand, ddraw};
                    }
                }
                p += len;
                ddraw += len;
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
    for (int o = 16; o > 0; o >>= 1) {
        screened += __shfl_down_sync(0xffffffffu, screened, o);
        exact += __shfl_down_sync(0xffffffffu, exact, o);
    }
    if ((tid & 31) == 0) {
        atomicAdd(&A.ctrl->screened, screened);
        atomicAdd(&A.ctrl->exact_evals, exact);
    }
    if (!tc_ok) atomicOr(&A.ctrl->err, kErrTc);
    __syncthreads();
    if (s_gbad[grp] != 0u && tg.issuer) (void)mbar_wait(tg.mbar, s_fail_phase[grp]);  // bounded
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tc_dealloc(s_tbase, 32);
}

using TcScreenFn = void (*)(TcScreenArgs);

TcScreenFn screen_tc_fn(bool fast_delta, bool fp16) {
    if (fast_delta) return fp16 ? screen_tc_kernel<true, true> : screen_tc_kernel<true, false>;
    return fp16 ? screen_tc_kernel<false, true> : screen_tc_kernel<false, false>;
}

// Survivor regeneration for the precision form: the key holds the FP64 score
// rounded to f32.
template <bool kFastDelta>
__global__ void regen64_kernel(const __grid_constant__ ScreenArgs A, const Entry *__restrict__ fin,
                               const unsigned long long *__restrict__ ids, const unsigned int *__restrict__ tribes,
                               csx_survivor *__restrict__ out) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.keep) return;
    const Entry e = fin[q];
    const bool real = e.k1 != 0ull;
    const bool next_real = (q + 1 < A.keep) ? (fin[q + 1].k1 != 0ull) : false;
    if (q == 0 && !real) A.ctrl->n_out = 0;
    if (real && !next_real) A.ctrl->n_out = q + 1;
    if (!real) return;
    const uint32_t item = ~static_cast<uint32_t>(e.k1);
    const uint32_t dcand = ~static_cast<uint32_t>(e.k2 >> 32);
    const uint32_t ddraw = static_cast<uint32_t>(e.k2);
    const Item it = A.items[item];
    const uint64_t seed_t = stream_seed(A.seed, it.stream);
    const uint64_t draw = it.draw0 + ddraw;
    const CandHead h = cand_head(A.sc, seed_t, draw);
    float genes[kNtot];
    (void)synth_score<kFastDelta, true>(A.m, A.sc, A.el, seed_t, draw, h, genes);
    const float s = static_cast<float>(score64_genes(A.m, genes));
    if (score_okey(s) != static_cast<unsigned int>(e.k1 >> 32)) atomicOr(&A.ctrl->err, kErrRegen);
    csx_survivor v;
    v.score = s;
    v.tribe = tribes[h.ea];
    v.pa = ids[h.ea];
    v.pb = ids[h.eb];
    v.stream = it.stream;
    v.index = it.idx0 + dcand;
    v.draw = draw;
#pragma unroll
    for (int k = 0; k < kNtot; ++k) v.g[k] = genes[k];
    v.reserved = 0;
    out[q] = v;
}

}  // namespace csx
