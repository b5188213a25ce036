// csx_screen.cu — the GB300 screen funnel: src/screen.zig:run as a pipeline
// of sm_103a kernels behind the C ABI of include/csx_screen.h. One
// translation unit; its parts:
//   csx_pipeline.cuh        types; item building (walk, link, assembly, items)
//   csx_screen_kernels.cuh  screen kernels, merge tree, regeneration
//   this file               host orchestration, the single-screen C ABI and
//                           the allocation-free entry point
//   csx_batch.cuh           batched islands
//   csx_precision.cuh       the precision form's model and csx_tc_score
//
// Work decomposition. The reference runs T splitmix64 streams, stream t
// producing my_t candidates sequentially (src/screen.zig:273-297). A
// candidate consumes 33, 35, 62 or 64 draws, so where candidate i starts in
// its stream is only known by walking the stream. The pipeline:
//
//  1. walk    one thread per segment of L draws: the chain of candidate
//             starts from the segment's first draw (a guess), a checkpoint
//             every D candidates.
//  2. link    one warp per segment boundary: this chain and the next
//             segment's guess chain advance in speculative runs until they
//             share a start; chains that share a start coincide from there on,
//             and stream t's first chain starts at draw 0 (the truth), so the
//             truth is carried from segment to segment at the meeting points.
//  3. assemble one CTA per stream: the true candidate range of every segment
//             and its stream-local start index (late meetings repaired locally).
//  4. scan + emit  work items of <= D candidates with known start draw and
//             stream-local index, in (stream, index) order.
//  5. screen  persistent CTAs pull items; each thread synthesises and scores
//             candidates in registers; those that beat the CTA's threshold go
//             to a shared-memory buffer that is merged into the CTA's sorted
//             top-K list (bitonic sort). HBM sees only items and survivors.
//  6. merge   a tree of pairwise bitonic merges reduces the CTA lists.
//  7. regen   the K survivors are re-synthesised from (stream, draw) to
//             recover genes and lineage; the score is re-checked bit for bit.
//
// The walk costs two hashes per candidate against ~62 for synthesis. When
// streams are no longer than one item, steps 1-4 are skipped.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "../../include/csx_screen.h"
#include "csx_device.cuh"
#include "csx_tc.cuh"
#include "csx_pipeline.cuh"
#include "csx_screen_kernels.cuh"
#include "csx_prune.cuh"
#include "csx_ties.cuh"

namespace csx {

// ---- host orchestration ------------------------------------------------------------

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(n, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
};

struct Context {
    std::mutex mu;
    bool init = false;
    int num_sms = 0;
    size_t max_smem = 0;
    cudaEvent_t done = nullptr;
    cudaEvent_t ev[6] = {};
    bool timed = false;
    csx_run_info info{};
    DevBuf genomes, tab, ids, tribes, recs, ck, segout, off, items, lists_a, lists_b, ctrl, surv,
        result, pub, tie_hits, tie_count, tie_streams, tie_out;
    // batched islands
    DevBuf batch, b_genomes, b_surv, b_result;
    void *pinned = nullptr;         // host staging of the island descriptors (page-locked)
    cudaEvent_t desc_ev = nullptr;  // the descriptors' copy has run
    bool desc_pending = false;
    cudaStream_t aux[64] = {};      // one forked stream per island for the item stages
    cudaEvent_t ev_fork = nullptr, ev_join[64] = {};
    cudaStream_t pst = nullptr;     // private stream of the host batch call
    cudaGraphExec_t gexec = nullptr;
    csx_batch_info binfo{};
    const Entry *fin = nullptr;  // final list of the last single screen (kpad entries)
    uint32_t fin_kpad = 0;
};

Context g_ctx[64];

// A decimal environment value, dflt when unset or not a number (an explicit 0
// is 0: for CSX_ITEM_CANDS / CSX_SEG_CANDS that means automatic, for
// CSX_PRUNE_MIN_CANDS prune at every size).
uint64_t env_u64(const char *name, uint64_t dflt) {
    const char *v = std::getenv(name);
    if (!v || !*v) return dflt;
    char *end = nullptr;
    const unsigned long long x = std::strtoull(v, &end, 10);
    return (end && *end == 0) ? x : dflt;
}

uint32_t pow2_at_least(uint64_t x) {
    uint32_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

// unit() < p  <=>  (next() >> 40) < thr  (unit is exact: k * 2^-24)
uint32_t unit_threshold(float prob) {
    if (!(prob > 0.0f)) return 0;  // also NaN: the comparison is always false
    if (prob >= 1.0f) return 1u << 24;
    const double x = std::ldexp(static_cast<double>(prob), 24);  // exact
    return static_cast<uint32_t>(std::ceil(x));
}

#define CSX_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            std::fprintf(stderr, "csx: %s failed: %s\n", #call, cudaGetErrorString(e_));     \
            return e_ == cudaErrorMemoryAllocation ? CSX_ERR_OOM : CSX_ERR_CUDA;               \
        }                                                                                     \
    } while (0)

struct Plan {
    StreamGeom g;
    bool short_path = false;
    uint64_t items_cap = 0;
    uint32_t kpad = 0, sort_n = 0, buf_cap = 0;
    int grid = 0;
    size_t smem = 0;
    bool fast_delta = true;
    bool filter = false;
    bool tc = false, fp16 = false;  // precision form (tensor cores + FP64 band)
    float err = 0.0f;
    JumpBound jb{};  // widening of err for a candidate with a jump (filter mode)
    bool prune = false;     // the pruning screen (csx_prune.cuh)
    bool prune_ok = false;  // its bound is certifiable for this call (the batch decides for itself)
    bool prune_tc = false;  // its bound's gradient on the tensor cores
    int nb = 16;            // crossover genes its bound draws
    bool el_smem = false;   // its elite table in shared memory (prune_el_smem)
    PruneConst pc{};
    PruneTc ptc{};
};

int context_init(Context &cx, int dev) {
    if (cx.init) return CSX_OK;
    int v = 0;
    CSX_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    cx.num_sms = v;
    CSX_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cx.max_smem = static_cast<size_t>(v);
    CSX_CUDA(cudaEventCreateWithFlags(&cx.done, cudaEventDisableTiming));
    for (auto &e : cx.ev) CSX_CUDA(cudaEventCreate(&e));
    cx.init = true;
    return CSX_OK;
}

using ScreenFn = void (*)(ScreenArgs);

ScreenFn screen_fn(bool fast_delta, bool filter) {
    if (fast_delta) return filter ? screen_q_kernel<true> : screen_kernel<true>;
    return filter ? screen_q_kernel<false> : screen_kernel<false>;
}

using FullScreenFn = void (*)(FullScreenArgs);

FullScreenFn screen_full_fn(bool fast_delta) {
    return fast_delta ? screen_kernel<true, FullScreenArgs> : screen_kernel<false, FullScreenArgs>;
}

FullModel make_full_model(const csx_model_full &m) {
    FullModel f;
    f.w0 = m.w0;
    for (int k = 0; k < kNtot; ++k) f.wlin[k] = m.w_lin[k];
    for (int q = 0; q < kNqFull; ++q) f.wq[q] = m.w_quad[q];
    return f;
}

// Shared memory of the plain screen: the sort buffer, the elite table and,
// in the filter form, the queue of candidates awaiting the exact order.
size_t screen_smem(uint32_t sort_n, int ne, bool filter) {
    return static_cast<size_t>(sort_n) * sizeof(Entry) + static_cast<size_t>(ne + 1) * kNtot * sizeof(float) +
           (filter ? kPendCap * sizeof(Pend) : 0);
}

template <typename Fn>
int screen_occupancy(Fn fn, int num_sms, size_t smem, int *blocks) {
    CSX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int nb = 0;
    CSX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, smem));
    *blocks = std::max(1, nb) * num_sms;
    return CSX_OK;
}

// Bound on |filter score - exact score| for genes in [0, 1]: the exact
// order puts each term through at most 35 roundings (2 products, 16 lane
// adds, the lane total, 15 reduction adds, the tail add), the FFMA form
// through at most 47 (16 Horner steps, 30 outer steps, slack one); a sum of
// terms evaluated with at most n roundings per term is within
// gamma_n * sum|terms| (gamma_n = n u / (1 - n u), u = 2^-24) of the real sum.
// Returns 0 when the filter cannot be used (non-finite or huge weights).
float filter_bound(const csx_model &m) {
    double a = 16.0 * std::fabs(static_cast<double>(m.w0));
    for (int k = 0; k < kNtot; ++k) a += std::fabs(static_cast<double>(m.w_lin[k]));
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) a += std::fabs(static_cast<double>(m.w_quad[i * 16 + j]));
    if (!std::isfinite(a) || a > 1e30) return 0.0f;
    const double u = std::ldexp(1.0, -24);
    auto gamma = [u](double n) { return n * u / (1.0 - n * u); };
    const double e = (gamma(35) + gamma(47)) * a * (1.0 + std::ldexp(1.0, -20)) + 1e-30;
    return std::nextafter(static_cast<float>(e), INFINITY);
}

// JumpBound of a model whose filter_bound is nonzero (finite weights): an
// upper bound on how far the real surface can rise when gene j moves within
// [0, 1] (only a rise can lift a candidate over the threshold). With δ = v -
// u the move and the other genes in [0, 1], the change is
// δ (w_j + Σ_{i≠j} Q_ij g_i) + Q_jj (v² - u²): at most max(0, a_hi) +
// max(0, Q_jj) for δ >= 0 and max(0, -a_lo) + max(0, -Q_jj) for δ < 0, where
// a_hi / a_lo add the positive / negative Q_ij to w_j. Computed in double and
// rounded up with a 2^-20 relative margin.
void jump_bound(const csx_model &m, JumpBound *jb) {
    for (int j = 0; j < 32; ++j) jb->c[j] = 0.0f;
    for (int j = 0; j < kNtot; ++j) {
        const double w = static_cast<double>(m.w_lin[j]);
        double a_hi = w, a_lo = w, qjj = 0.0;
        if (j < 16) {
            for (int i = 0; i < 16; ++i) {  // row j (i <= j) and column j (i > j) of the triangle
                const double q = static_cast<double>(i <= j ? m.w_quad[j * 16 + i] : m.w_quad[i * 16 + j]);
                if (i == j) qjj = q;
                else if (q > 0.0) a_hi += q;
                else a_lo += q;
            }
        }
        const double up = std::max(0.0, a_hi) + std::max(0.0, qjj);
        const double down = std::max(0.0, -a_lo) + std::max(0.0, -qjj);
        const double c = std::max(up, down) * (1.0 + std::ldexp(1.0, -20));
        jb->c[j] = c > 0.0 ? std::nextafter(static_cast<float>(c), INFINITY) : 0.0f;
    }
}

// The generation's stream split (src/screen.zig:267-297) and the range
// [t_begin, t_end) of it this call screens (t_end = 0: every stream).
int split_streams(const csx_cfg &cfg, uint64_t t_begin, uint64_t t_end, StreamGeom &g) {
    g.seed = cfg.seed;
    g.T = std::max<uint64_t>(1, std::min<uint64_t>(cfg.threads, cfg.lambda));  // src/screen.zig:267
    g.per = cfg.lambda / g.T;
    g.my_last = cfg.lambda - (g.T - 1) * g.per;
    if (g.T >= 0xFFFFFFFFull) return CSX_ERR_LIMIT;
    g.link_cap = env_u64("CSX_LINK_CAP", kLinkCap);  // a lower cap makes the link's failure path testable
    if (t_end == 0) t_end = g.T;  // the whole generation
    if (t_begin >= t_end || t_end > g.T) return CSX_ERR_BAD_ARGS;
    g.t0 = t_begin;
    g.nT = t_end - t_begin;
    return CSX_OK;
}

// Entries of a CTA list: the next power of two above K, so K + 1 entries for K
// <= 2048 (the final (K+1)-th entry shows a tie at the K-th score: fix_ties).
uint32_t list_kpad(uint64_t keep) {
    return std::max<uint32_t>(32, pow2_at_least(keep + (keep <= 2048 ? 1 : 0)));
}

// Mutation form, filter bounds and the CTA list / buffer sizes of a plan.
void screen_shape(const csx_cfg &cfg, const csx_model &model, bool full, Plan *pl) {
    pl->fast_delta = std::isfinite(cfg.sigma) && std::fabs(cfg.sigma) <= 1.0e38f &&
                     (cfg.sigma == 0.0f || std::fabs(cfg.sigma) >= 1.0e-30f);
    pl->err = filter_bound(model);
    jump_bound(model, &pl->jb);
    pl->filter = !full && !(cfg.flags & CSX_FLAG_EXACT_ALL) && pl->err > 0.0f;
    // the pruning screen: the filter form's conditions, the fast delta form
    // (its mutation is within |sigma| of the parent gene by construction) and
    // a certifiable bound. The precision form (TC flags) prunes with its tile
    // format's bound and ranks in FP64; without a tensor-core bound it keeps
    // its own unpruned kernel.
    const uint32_t tcf = cfg.flags & (CSX_FLAG_TC_BF16 | CSX_FLAG_TC_FP16);
    pl->prune = pl->filter && pl->fast_delta && !(cfg.flags & CSX_FLAG_NO_PRUNE) &&
                make_prune(model, cfg.sigma, &pl->pc, &pl->nb);
    pl->prune_tc = pl->prune && (tcf != 0 || !(cfg.flags & CSX_FLAG_PRUNE_FFMA)) &&
                   make_prune_tc(model, pl->pc, tcf != CSX_FLAG_TC_BF16, &pl->ptc);
    if (tcf && !pl->prune_tc) pl->prune = false;
    pl->kpad = list_kpad(cfg.keep);
    pl->sort_n = pow2_at_least(pl->kpad + 4ull * kThreads);
    pl->buf_cap = pl->sort_n - pl->kpad;
}

// Walk segments of about `seg` candidates (g.d_log2 set): L draws rounded to
// the candidate length when it is constant, the segment counts, and a
// checkpoint capacity (below).
//
// Candidates past its own end that a segment's truth range reaches before its
// chain meets the next segment's (the link's walk), simulated over 30000
// random boundaries of the reference's length rule (62 / 64 / 33 / 35 draws,
// immigrant 1%, jump 2%): median 136, 99th percentile 11.9k, 99.99th 24.1k,
// largest 27.5k. The pooled plan's checkpoints cover at least the segment plus
// this margin, so short segments keep their items at D candidates; past the
// last checkpoint a segment's final item grows instead (correct, but one
// thread screens it alone: a margin of 24576 left a few such items per island
// of the batched workload and slowed it by a fifth).
constexpr uint64_t kLinkSlackCands = 65536;

// Checkpoints of a segment: one per D starts over `L / 33` starts (every
// candidate 33 draws long), and with `slack` at least over the segment's
// nominal candidates plus kLinkSlackCands.
void segment_geometry(const csx_cfg &cfg, uint64_t seg, bool slack, StreamGeom &g) {
    const uint64_t my_max = std::max(g.per, g.my_last);
    const bool has_last = g.t0 + g.nT == g.T;
    // candidate length is constant when neither branch probability is mixed
    const uint32_t it = unit_threshold(cfg.imm_p), jt = unit_threshold(cfg.jump_p);
    uint64_t gran = 2;
    if ((it == 0 || it == (1u << 24)) && (jt == 0 || jt == (1u << 24)))
        gran = (it ? 33 : 62) + (jt ? 2 : 0);
    uint64_t L = 64 * std::min(std::min<uint64_t>(seg, 1ull << 24), my_max);  // <= 2^30 draws (walk_kernel)
    L = ((L + gran - 1) / gran) * gran;
    g.L = L;
    g.C = static_cast<uint32_t>(std::max<uint64_t>(1, (64 * g.per + L - 1) / L));
    g.C_last = static_cast<uint32_t>(std::max<uint64_t>(1, (64 * g.my_last + L - 1) / L));
    g.n_seg = (g.nT - 1) * g.C + (has_last ? g.C_last : g.C);
    uint64_t cover = L / 33;  // starts if every candidate were 33 draws long
    if (slack) cover = std::max<uint64_t>(cover, std::min(seg, my_max) + kLinkSlackCands);
    g.ckcap = static_cast<uint32_t>(cover / (1ull << g.d_log2) + 3);
}

// A share of one generation's work items (csx_screen_items): every share
// builds the same item list and screens its part of it.
struct Shard {
    uint32_t index = 0, count = 1;
};

// grid_override, item_cands, seg_cands: 0 = automatic (the batched screen
// passes its own grid and the tuner's sizes). A sharded call sizes its items
// by a fixed SM count, so that every share's item list is the same whatever
// GPU it runs on.
constexpr int kItemRefSms = 152;

int make_plan(const Context &cx, const csx_cfg &cfg, const csx_model &model, int ne, Plan *pl,
              int grid_override = 0, uint64_t item_cands = 0, uint64_t seg_cands = 0, uint64_t t_begin = 0,
              uint64_t t_end = 0, const csx_model_full *full = nullptr, bool sharded = false) {
    StreamGeom &g = pl->g;
    int src = split_streams(cfg, t_begin, t_end, g);
    if (src) return src;
    const uint64_t my_max = std::max(g.per, g.my_last);
    const bool has_last = g.t0 + g.nT == g.T;
    const uint64_t lam_range = (g.nT - (has_last ? 1 : 0)) * g.per + (has_last ? g.my_last : 0);
    screen_shape(cfg, model, full != nullptr, pl);
    const uint32_t tcf = cfg.flags & (CSX_FLAG_TC_BF16 | CSX_FLAG_TC_FP16);
    if (tcf == (CSX_FLAG_TC_BF16 | CSX_FLAG_TC_FP16)) return CSX_ERR_BAD_ARGS;
    if (full && tcf) return CSX_ERR_BAD_ARGS;  // the precision form scores the reference surface
    pl->tc = tcf != 0;  // FP64 ranking (pruned, or the unpruned precision kernel)
    pl->fp16 = tcf == CSX_FLAG_TC_FP16;
    // pruning pays once the generation gives each screen thread a few hundred
    // candidates (the threshold then settles early; measured against the
    // unpruned filter kernel: 0.40 against 0.29 ms at 1e6, 0.78 against 0.54
    // at 1e7, 1.35 against 1.21 at 3e7, 3.14 against 3.45 at 1e8 candidates):
    // prune from 400 per thread of a three-CTA-per-SM grid
    const uint64_t sms = sharded ? kItemRefSms : static_cast<uint64_t>(cx.num_sms);
    const uint64_t min_prune = env_u64("CSX_PRUNE_MIN_CANDS", 400ull * 3 * sms * kThreads);
    pl->prune_ok = pl->prune && lam_range >= min_prune;
    if (pl->prune_ok && grid_override == 0) {
        // the selection scratch holds one key per CTA: at most 8 CTAs of 256 threads per SM
        pl->el_smem = prune_el_smem(pl->sort_n, ne, pl->nb, cx.num_sms, pl->prune_tc, cx.max_smem);
        pl->smem = prune_smem(pl->sort_n, ne, pl->nb, cx.num_sms, pl->prune_tc, pl->el_smem);
        pl->prune = pl->smem + 1024 <= cx.max_smem;
    } else {
        pl->prune = false;
    }
    if (!pl->prune)
        pl->smem = pl->tc ? static_cast<size_t>(pl->sort_n) * sizeof(Entry) +
                                static_cast<size_t>(ne + 1) * kNtot * sizeof(float) + kTcSmemExtra
                          : screen_smem(pl->sort_n, ne, pl->filter);
    if (pl->smem + 1024 > cx.max_smem) return CSX_ERR_LIMIT;
    if (grid_override > 0) {
        pl->grid = grid_override;
    } else if (pl->prune) {
        int rc = screen_occupancy(screen_p_fn(pl->nb, pl->prune_tc, pl->fp16 || !pl->tc, pl->tc), cx.num_sms,
                                  pl->smem, &pl->grid);
        if (rc) return rc;
        // The occupancy query reports one CTA per SM for the tensor-core form;
        // its registers (80 at three CTAs), shared memory (~65 KB each) and
        // TMEM (32 columns each) hold three, which run 9% faster than two
        // (measured). The screen is persistent with dynamic work, so any grid
        // is correct.
        if (pl->prune_tc) {
            const int fit = static_cast<int>((228u << 10) / (pl->smem + 1024));  // 228 KB of shared memory per SM
            pl->grid = std::max(pl->grid, std::min(3, std::max(1, fit)) * cx.num_sms);
        }
    } else if (pl->tc) {
        // The occupancy query reports one CTA per SM for this kernel, yet three
        // are resident and run faster (80 registers, ~50 KB of shared memory,
        // 32 TMEM columns each; measured). The screen is persistent with
        // dynamic work, so any grid is correct: launch three per SM.
        int rc = screen_occupancy(screen_tc_fn(pl->fast_delta, pl->fp16), cx.num_sms, pl->smem, &pl->grid);
        if (rc) return rc;
        pl->grid = kTcCtasPerSm * cx.num_sms;
    } else if (full) {
        int rc = screen_occupancy(screen_full_fn(pl->fast_delta), cx.num_sms, pl->smem, &pl->grid);
        if (rc) return rc;
    } else {
        int rc = screen_occupancy(screen_fn(pl->fast_delta, pl->filter), cx.num_sms, pl->smem, &pl->grid);
        if (rc) return rc;
    }

    // item size D: about 64 items per thread of a three-CTA-per-SM grid, set
    // by the GPU's size rather than the kernel's grid (measured: smaller items
    // shorten the tail of the persistent grid more than their reads cost; at
    // 2.65e9, 256 candidates beat 512 by 0.5% with three CTAs per SM and by
    // 0.25% with the filter kernel's two)
    uint64_t d = item_cands ? item_cands : env_u64("CSX_ITEM_CANDS", 0);
    if (d == 0) {
        const uint64_t target = 64ull * 3 * static_cast<uint64_t>(sharded ? kItemRefSms : cx.num_sms) * kThreads;
        d = std::max<uint64_t>(1, lam_range / target);
        d = std::min<uint64_t>(16384, std::max<uint64_t>(64, d));
    }
    // the link's speculative runs hold up to 32 starts and record at most one
    // checkpoint each, so checkpoints (and items) stay at least 64 apart
    d = std::max<uint64_t>(64, d);
    uint32_t dl = 0;
    while ((2ull << dl) <= d) ++dl;  // D = 2^dl <= d
    g.d_log2 = dl;
    const uint64_t D = 1ull << dl;
    // walk segments of about sqrt(lambda) candidates, within [1024, 49152]:
    // the walk is serial within a segment (its time grows with the segment)
    // and the link costs about the same per boundary (its total grows with
    // lambda / segment), so the sum is least near sqrt(lambda) times a
    // constant; measured optima: 1024 at 1e6 (items 0.70 ms, 5.1 at 49152),
    // 12288 at 2e8 (2.56 ms; 3.47 at 5139, 5.68 at 49152), 49152 at 2.65e9.
    // It depends on lambda only, so every share of a sharded call builds the
    // same segments.
    uint64_t seg = seg_cands ? seg_cands : env_u64("CSX_SEG_CANDS", 0);
    if (seg == 0) {
        uint64_t r = static_cast<uint64_t>(std::sqrt(static_cast<double>(lam_range)));
        while (r * r > lam_range) --r;
        while ((r + 1) * (r + 1) <= lam_range) ++r;
        seg = std::min<uint64_t>(kDefaultSegCands, std::max<uint64_t>(1024, r));
    }
    segment_geometry(cfg, seg, true, g);
    pl->short_path = my_max <= D;
    // a segment's range of cnt candidates splits at the multiples of D inside
    // it: at most 2 + cnt / D items, and the ranges partition the candidates
    pl->items_cap = pl->short_path ? g.nT : 2 * g.n_seg + lam_range / D + 1;
    if (pl->items_cap >= 0xFFFFFFFFull) return CSX_ERR_LIMIT;
    return CSX_OK;
}

int unit_blocks(uint64_t n, int threads) { return static_cast<int>((n + threads - 1) / threads); }

SynthConst make_synth(const csx_cfg &cfg, int ne) {
    SynthConst sc;
    sc.ne = static_cast<uint32_t>(ne);
    sc.ne_magic = ~0ull / static_cast<uint64_t>(ne) + 1;
    sc.imm_thr = unit_threshold(cfg.imm_p);
    sc.jump_thr = unit_threshold(cfg.jump_p);
    sc.sigma = cfg.sigma;
    sc.nsig1 = -cfg.sigma;
    sc.sigma23 = cfg.sigma * 0x1p-23f;
    return sc;
}

DevModel make_dev_model(const csx_model &model) {
    DevModel m;
    m.w0 = model.w0;
    m.w16 = 16.0f * model.w0;
    for (int k = 0; k < kNtot; ++k) m.wlin[k] = model.w_lin[k];
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) m.wq[tri(i, j)] = model.w_quad[i * 16 + j];
    m.tail = 0u;
    for (int k = 16; k < kNtot; ++k) m.tail |= model.w_lin[k] != 0.0f ? 1u : 0u;  // NaN counts as nonzero
    return m;
}

// The item-building stages on `st` (walk, link, assembly, scan, emit), or one
// item per stream when every stream fits in one item. recs / ck / so / off
// are unused on the short path.
int enqueue_items(const SynthConst &sc, const Plan &pl, SegRec *recs, uint64_t *ck, SegOut *so, uint32_t *off,
                  Item *items, Ctrl *ctrl, cudaStream_t st, uint32_t *launches) {
    const StreamGeom &g = pl.g;
    if (pl.short_path) {
        stream_items_kernel<<<unit_blocks(g.nT, 256), 256, 0, st>>>(g, items, ctrl);
        CSX_CUDA(cudaGetLastError());
        ++*launches;
        return CSX_OK;
    }
    walk_kernel<<<unit_blocks(g.n_seg, 128), 128, 0, st>>>(sc, g, recs, ck, ctrl);
    CSX_CUDA(cudaGetLastError());
    link_kernel<<<unit_blocks(g.n_seg * 32, 128), 128, 0, st>>>(sc, g, recs, ck, ctrl);
    CSX_CUDA(cudaGetLastError());
    if (g.C >= 64)
        assemble_block_kernel<<<static_cast<unsigned>(g.nT), kAsmThreads, 0, st>>>(g, recs, so, ctrl);
    else
        assemble_kernel<<<unit_blocks(g.nT, 128), 128, 0, st>>>(g, recs, so, ctrl);
    CSX_CUDA(cudaGetLastError());
    scan_kernel<<<1, 1024, 0, st>>>(so, g.n_seg, off, ctrl, pl.items_cap);
    CSX_CUDA(cudaGetLastError());
    emit_kernel<<<unit_blocks(g.n_seg, 128), 128, 0, st>>>(g, so, off, ck, items, ctrl);
    CSX_CUDA(cudaGetLastError());
    *launches += 5;
    return CSX_OK;
}

// The screen's arguments for a plan (the reference surface's model slot set).
ScreenArgs screen_args(const csx_cfg &cfg, const csx_model &model, const SynthConst &sc, const Plan &pl,
                       const float *tab, const Item *items, Ctrl *ctrl, Entry *lists) {
    ScreenArgs A;
    A.m = make_dev_model(model);
    A.sc = sc;
    A.seed = cfg.seed;
    A.el = tab;
    A.items = items;
    A.ctrl = ctrl;
    A.lists = lists;
    A.keep = static_cast<uint32_t>(cfg.keep);
    A.kpad = pl.kpad;
    A.sort_n = pl.sort_n;
    A.buf_cap = pl.buf_cap;
    A.err = pl.err;
    A.jb = pl.jb;
    return A;
}

// Merge tree of nl CTA lists (kpad entries each) between the two buffers;
// *fin receives the buffer holding the final list.
int enqueue_merge(Entry *cur, Entry *nxt, uint32_t nl, uint32_t kpad, cudaStream_t st, Entry **fin,
                  uint32_t *launches) {
    const size_t msmem = 2ull * kpad * sizeof(Entry);
    CSX_CUDA(cudaFuncSetAttribute(merge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(msmem)));
    uint32_t n = nl;
    while (n > 1) {
        const uint32_t m = (n + 1) / 2;
        merge_kernel<<<m, 256, msmem, st>>>(cur, n, nxt, kpad);
        CSX_CUDA(cudaGetLastError());
        ++*launches;
        std::swap(cur, nxt);
        n = m;
    }
    *fin = cur;
    return CSX_OK;
}

// Enqueue the whole pipeline on `st`. Device inputs: genomes (csx_genome x ne).
int enqueue_screen(Context &cx, const csx_cfg &cfg, const csx_model &model, const csx_genome *d_genomes,
                   int ne, csx_survivor *d_out, unsigned long long *d_result, cudaStream_t st,
                   uint64_t t_begin = 0, uint64_t t_end = 0, const csx_model_full *full = nullptr,
                   Shard shard = Shard{}) {
    Plan pl;
    int rc = make_plan(cx, cfg, model, ne, &pl, 0, 0, 0, t_begin, t_end, full, shard.count > 1);
    if (rc) return rc;
    const StreamGeom &g = pl.g;
    const bool fast = pl.fast_delta;

    CSX_CUDA(cx.tab.ensure(static_cast<size_t>(ne + 1) * kNtot * sizeof(float)));
    CSX_CUDA(cx.ids.ensure(static_cast<size_t>(ne) * sizeof(unsigned long long)));
    CSX_CUDA(cx.tribes.ensure(static_cast<size_t>(ne) * sizeof(unsigned int)));
    CSX_CUDA(cx.ctrl.ensure(sizeof(Ctrl)));
    CSX_CUDA(cx.items.ensure(pl.items_cap * sizeof(Item)));
    const uint32_t nl = static_cast<uint32_t>(pl.grid);
    CSX_CUDA(cx.lists_a.ensure(static_cast<size_t>(nl) * pl.kpad * sizeof(Entry)));
    CSX_CUDA(cx.lists_b.ensure(static_cast<size_t>((nl + 1) / 2) * pl.kpad * sizeof(Entry)));
    if (pl.prune) CSX_CUDA(cx.pub.ensure(static_cast<size_t>(kPruneMs) * nl * sizeof(uint32_t)));
    if (!pl.short_path) {
        CSX_CUDA(cx.recs.ensure(g.n_seg * sizeof(SegRec)));
        CSX_CUDA(cx.ck.ensure(g.n_seg * g.ckcap * sizeof(uint64_t)));
        CSX_CUDA(cx.segout.ensure(g.n_seg * sizeof(SegOut)));
        CSX_CUDA(cx.off.ensure(g.n_seg * sizeof(uint32_t)));
    }
    Ctrl *ctrl = static_cast<Ctrl *>(cx.ctrl.p);
    CSX_CUDA(cudaStreamWaitEvent(st, cx.done, 0));
    cx.timed = (cfg.flags & CSX_FLAG_STAGE_TIMES) != 0;
    cx.info = csx_run_info{};
    cx.info.screen_ctas = static_cast<uint32_t>(pl.grid);
    cx.info.segments = pl.short_path ? 0 : g.n_seg;
    cx.info.seg_draws = pl.short_path ? 0 : g.L;
    cx.info.item_cands = 1ull << g.d_log2;
    uint32_t launches = 0;
    auto mark = [&](int i) -> cudaError_t { return cx.timed ? cudaEventRecord(cx.ev[i], st) : cudaSuccess; };
    CSX_CUDA(mark(0));
    CSX_CUDA(cudaMemsetAsync(ctrl, 0, sizeof(Ctrl), st));
    if (pl.prune) CSX_CUDA(cudaMemsetAsync(cx.pub.p, 0, static_cast<size_t>(kPruneMs) * nl * sizeof(uint32_t), st));

    const SynthConst sc = make_synth(cfg, ne);

    float *tab = static_cast<float *>(cx.tab.p);
    auto *ids = static_cast<unsigned long long *>(cx.ids.p);
    auto *tribes = static_cast<unsigned int *>(cx.tribes.p);
    prep_elites_kernel<<<unit_blocks(static_cast<uint64_t>(ne + 1) * kNtot, 256), 256, 0, st>>>(
        d_genomes, ne, tab, ids, tribes);
    CSX_CUDA(cudaGetLastError());
    ++launches;
    CSX_CUDA(mark(1));

    Item *items = static_cast<Item *>(cx.items.p);
    rc = enqueue_items(sc, pl, static_cast<SegRec *>(cx.recs.p), static_cast<uint64_t *>(cx.ck.p),
                       static_cast<SegOut *>(cx.segout.p), static_cast<uint32_t *>(cx.off.p), items, ctrl, st,
                       &launches);
    if (rc) return rc;
    if (shard.count > 1) {
        shard_items_kernel<<<1, 32, 0, st>>>(ctrl, shard.index, shard.count);
        CSX_CUDA(cudaGetLastError());
        ++launches;
    }
    CSX_CUDA(mark(2));

    const ScreenArgs A = screen_args(cfg, model, sc, pl, tab, items, ctrl, static_cast<Entry *>(cx.lists_a.p));
    if (pl.prune) {
        PruneArgs P;
        static_cast<ScreenArgs &>(P) = A;
        P.pc = pl.pc;
        P.tc = pl.ptc;
        P.pub = static_cast<uint32_t *>(cx.pub.p);
        P.sel_cap = 8u * static_cast<uint32_t>(cx.num_sms);
        P.el_smem = pl.el_smem ? 1u : 0u;
        screen_p_fn(pl.nb, pl.prune_tc, pl.fp16 || !pl.tc, pl.tc)<<<pl.grid, kThreads, pl.smem, st>>>(P);
    } else if (pl.tc) {
        TcScreenArgs P;
        P.A = A;
        P.band = kTcBand;
        rc = make_tc_model(model, pl.fp16, &P.tm);
        if (rc) return rc;
        rc = tc_error_bound(model, pl.fp16, &P.err_abs);
        if (rc) return rc;
        screen_tc_fn(fast, pl.fp16)<<<pl.grid, kThreads, pl.smem, st>>>(P);
    } else if (full) {
        FullScreenArgs F;
        static_cast<ScreenArgs &>(F) = A;
        F.fm = make_full_model(*full);
        screen_full_fn(fast)<<<pl.grid, kThreads, pl.smem, st>>>(F);
    } else {
        screen_fn(fast, pl.filter)<<<pl.grid, kThreads, pl.smem, st>>>(A);
    }
    CSX_CUDA(cudaGetLastError());
    ++launches;
    CSX_CUDA(mark(3));

    Entry *cur = nullptr;
    rc = enqueue_merge(static_cast<Entry *>(cx.lists_a.p), static_cast<Entry *>(cx.lists_b.p), nl, pl.kpad, st,
                       &cur, &launches);
    if (rc) return rc;
    cx.fin = cur;
    cx.fin_kpad = pl.kpad;
    CSX_CUDA(mark(4));
    if (full) {
        FullScreenArgs F;
        static_cast<ScreenArgs &>(F) = A;
        F.fm = make_full_model(*full);
        if (fast)
            regen_full_kernel<true><<<unit_blocks(cfg.keep, 128), 128, 0, st>>>(F, cur, ids, tribes, d_out);
        else
            regen_full_kernel<false><<<unit_blocks(cfg.keep, 128), 128, 0, st>>>(F, cur, ids, tribes, d_out);
    } else if (pl.tc && fast)
        regen64_kernel<true><<<unit_blocks(cfg.keep, 128), 128, 0, st>>>(A, cur, ids, tribes, d_out);
    else if (pl.tc)
        regen64_kernel<false><<<unit_blocks(cfg.keep, 128), 128, 0, st>>>(A, cur, ids, tribes, d_out);
    else if (fast)
        regen_kernel<true><<<unit_blocks(cfg.keep, 128), 128, 0, st>>>(A, cur, ids, tribes, d_out, d_result);
    else
        regen_kernel<false><<<unit_blocks(cfg.keep, 128), 128, 0, st>>>(A, cur, ids, tribes, d_out, d_result);
    CSX_CUDA(cudaGetLastError());
    result_kernel<<<1, 32, 0, st>>>(ctrl, d_result);
    CSX_CUDA(cudaGetLastError());
    launches += 2;
    CSX_CUDA(mark(5));
    cx.info.launches = launches;
    CSX_CUDA(cudaEventRecord(cx.done, st));
    return CSX_OK;
}

int check_common(const csx_cfg *cfg, const csx_model *model, int ne) {
    if (!cfg || !model) return CSX_ERR_BAD_ARGS;
    if (ne < 2) return CSX_ERR_NEED_TWO_ELITES;  // src/screen.zig:266
    if (cfg->keep == 0) return CSX_ERR_BAD_ARGS;  // Heap.offer would read slots[0] of an empty heap
    if (cfg->keep > kMaxKeep || static_cast<uint32_t>(ne) > kMaxElites) return CSX_ERR_LIMIT;
    return CSX_OK;
}

int current_context(Context **out) {
    int dev = 0;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return CSX_ERR_NO_DEVICE;
    }
    CSX_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return CSX_ERR_LIMIT;
    *out = &g_ctx[dev];
    return CSX_OK;
}

}  // namespace csx


using namespace csx;

extern "C" {

int csx_last_run_info(csx_run_info *out) {
    if (!out) return CSX_ERR_BAD_ARGS;
    Context *cx = nullptr;
    int rc = current_context(&cx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(cx->mu);
    *out = cx->info;
    if (cx->init && cx->timed) {
        CSX_CUDA(cudaEventSynchronize(cx->ev[5]));
        float *ms[5] = {&out->ms_prep, &out->ms_items, &out->ms_screen, &out->ms_merge, &out->ms_regen};
        for (int i = 0; i < 5; ++i) CSX_CUDA(cudaEventElapsedTime(ms[i], cx->ev[i], cx->ev[i + 1]));
        CSX_CUDA(cudaEventElapsedTime(&out->ms_total, cx->ev[0], cx->ev[5]));
        Ctrl c;
        CSX_CUDA(cudaMemcpy(&c, cx->ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost));
        out->exact_evals = c.exact_evals;
    }
    return CSX_OK;
}

int csx_limits(uint64_t *max_keep, uint64_t *max_elites) {
    if (max_keep) *max_keep = kMaxKeep;
    if (max_elites) *max_elites = kMaxElites;
    return CSX_OK;
}

}  // extern "C"

namespace csx {

int screen_device(const csx_cfg *cfg, const csx_model *model, const csx_genome *d_elites, int n_elites,
                  csx_survivor *d_out, uint64_t out_cap, uint64_t *d_result, void *cuda_stream,
                  const csx_model_full *full) {
    int rc = check_common(cfg, model, n_elites);
    if (rc) return rc;
    if (!d_elites || !d_result || (!d_out && cfg->lambda > 0)) return CSX_ERR_BAD_ARGS;
    if (out_cap < std::min<uint64_t>(cfg->keep, cfg->lambda)) return CSX_ERR_BAD_ARGS;
    Context *cx = nullptr;
    rc = current_context(&cx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(cx->mu);
    int dev = 0;
    CSX_CUDA(cudaGetDevice(&dev));
    rc = context_init(*cx, dev);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    if (cfg->lambda == 0) {  // one empty stream: nothing screened, nothing kept
        CSX_CUDA(cudaStreamWaitEvent(st, cx->done, 0));
        CSX_CUDA(cudaMemsetAsync(d_result, 0, 4 * sizeof(uint64_t), st));
        CSX_CUDA(cudaEventRecord(cx->done, st));
        return CSX_OK;
    }
    csx_cfg c = *cfg;
    return enqueue_screen(*cx, c, *model, d_elites, n_elites, d_out,
                          reinterpret_cast<unsigned long long *>(d_result), st, 0, 0, full);
}

const csx_model kZeroModel{};  // the reference surface's slot when the full surface scores

}  // namespace csx

extern "C" {

int csx_screen_device(const csx_cfg *cfg, const csx_model *model, const csx_genome *d_elites, int n_elites,
                      csx_survivor *d_out, uint64_t out_cap, uint64_t *d_result, void *cuda_stream) {
    return screen_device(cfg, model, d_elites, n_elites, d_out, out_cap, d_result, cuda_stream, nullptr);
}

int csx_model_full_from_compact(const float *w, int n, csx_model_full *out) {
    if (!w || !out) return CSX_ERR_BAD_ARGS;
    if (n != CSX_FULL_NF) return CSX_ERR_BAD_MODEL;
    out->w0 = w[0];
    for (int k = 0; k < kNtot; ++k) out->w_lin[k] = w[1 + k];
    for (int q = 0; q < kNqFull; ++q) out->w_quad[q] = w[1 + kNtot + q];
    return CSX_OK;
}

int csx_screen_full_device(const csx_cfg *cfg, const csx_model_full *model, const csx_genome *d_elites,
                           int n_elites, csx_survivor *d_out, uint64_t out_cap, uint64_t *d_result,
                           void *cuda_stream) {
    if (!model) return CSX_ERR_BAD_ARGS;
    return screen_device(cfg, &kZeroModel, d_elites, n_elites, d_out, out_cap, d_result, cuda_stream, model);
}

}  // extern "C"

namespace csx {

// ---- exact tie order (host half; device half in csx_ties.cuh) ----------------

uint32_t host_okey(float x) {
    x = x + 0.0f;  // -0 ranks with +0
    if (x != x) return 0u;
    uint32_t b;
    std::memcpy(&b, &x, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Heap.offer, src/screen.zig:166-192: a K-slot binary min-heap of f32 scores
// that rejects a score <= its root once full; slot order is the array order.
void tie_heap_offer(std::vector<TieHit> &h, size_t k, const TieHit &s) {
    if (h.size() < k) {
        h.push_back(s);
        size_t i = h.size() - 1;
        while (i > 0) {
            const size_t par = (i - 1) / 2;
            if (h[par].score <= h[i].score) break;
            std::swap(h[par], h[i]);
            i = par;
        }
        return;
    }
    if (s.score <= h[0].score) return;
    h[0] = s;
    size_t i = 0;
    for (;;) {
        const size_t l = 2 * i + 1, r = 2 * i + 2;
        size_t m = i;
        if (l < k && h[l].score < h[m].score) m = l;
        if (r < k && h[r].score < h[m].score) m = r;
        if (m == i) break;
        std::swap(h[m], h[i]);
        i = m;
    }
}

// The survivors out[0..cnt) of a whole-stream call, reordered as the
// reference orders them: the stable sort by score of the concatenated
// per-stream heaps (src/screen.zig:306-319). The screen ranks equal scores
// by (stream, index); that differs only inside a stream that holds two
// survivors of one f32 score, or a survivor at the K-th score (where the
// heap's history decides which tied candidates it kept). Such a stream's
// heap is replayed exactly: a candidate enters it only if it scores above
// the root, and the root only grows, so the stream is read in chunks of
// doubling length, each collecting (on the GPU, reference-order scores) the
// candidates above the root the previous chunks left, and the host offers
// them in index order to a heap with the reference's rules. The final list
// is the top cnt of those heaps and the other streams' survivors by (score
// descending, stream, heap slot); candidates taken from the replayed heaps
// are regenerated on the GPU. The precision form (FP64 ranking) has no
// reference counterpart and keeps (stream, index).
// The device buffers a finished screen left behind: its elite table, work
// items (n_items of them), ids and tribes.
struct ScreenBufs {
    const float *tab;
    const Item *items;
    uint64_t n_items;
    const unsigned long long *ids;
    const unsigned int *tribes;
    const Entry *fin;  // the final top-kpad list (its entry past the survivors shows a tie at the K-th score)
    uint32_t kpad;
};

int fix_ties(Context &cx, const csx_cfg &cfg, const csx_model &model, const csx_model_full *full, int ne,
             uint64_t t_begin, uint64_t t_end, csx_survivor *out, uint64_t cnt, const ScreenBufs &bufs,
             cudaStream_t st) {
    const uint64_t n_items = bufs.n_items;
    if (cnt == 0) return CSX_OK;
    const uint32_t tau = host_okey(out[cnt - 1].score);
    // a candidate outside the survivors ties with the K-th score when the
    // final list's next entry does (the lists keep K + 1 entries, and every
    // candidate scoring at least the running threshold entered them)
    bool boundary = false;
    if (cnt < bufs.kpad && bufs.fin) {
        Entry next{};
        CSX_CUDA(cudaMemcpyAsync(&next, bufs.fin + cnt, sizeof(Entry), cudaMemcpyDeviceToHost, st));
        CSX_CUDA(cudaStreamSynchronize(st));
        boundary = next.k1 != 0ull && static_cast<uint32_t>(next.k1 >> 32) == tau;
    }
    std::set<uint64_t> S;
    std::map<std::pair<uint64_t, uint32_t>, int> seen;
    for (uint64_t q = 0; q < cnt; ++q) {
        const uint32_t ok = host_okey(out[q].score);
        if (boundary && ok == tau) S.insert(out[q].stream);
        if (++seen[{out[q].stream, ok}] == 2) S.insert(out[q].stream);
    }
    if (S.empty()) return CSX_OK;
    Plan pl;
    int rc = make_plan(cx, cfg, model, ne, &pl, 0, 0, 0, t_begin, t_end, full);
    if (rc) return rc;
    const StreamGeom &g = pl.g;
    const SynthConst sc = make_synth(cfg, ne);
    const ScreenArgs A = screen_args(cfg, model, sc, pl, bufs.tab, bufs.items, nullptr, nullptr);
    FullScreenArgs F;
    static_cast<ScreenArgs &>(F) = A;
    if (full) F.fm = make_full_model(*full);
    const unsigned int cap = 1u << 20;
    CSX_CUDA(cx.tie_hits.ensure(static_cast<size_t>(cap) * sizeof(TieHit)));
    CSX_CUDA(cx.tie_count.ensure(sizeof(unsigned int)));
    auto *d_hits = static_cast<TieHit *>(cx.tie_hits.p);
    auto *d_count = static_cast<unsigned int *>(cx.tie_count.p);
    const int blocks = static_cast<int>(std::min<uint64_t>((n_items + 255) / 256, 32ull * cx.num_sms));
    const size_t K = static_cast<size_t>(cfg.keep);
    std::map<uint64_t, std::vector<TieHit>> heaps;
    std::vector<TieHit> hits;
    for (uint64_t t : S) {
        const uint64_t n_t = (t == g.T - 1) ? g.my_last : g.per;
        std::vector<TieHit> &h = heaps[t];
        uint64_t lo = 0, size = std::max<uint64_t>(4 * K, 1024);
        bool all = true;
        float thr = -INFINITY;
        while (lo < n_t) {
            const uint64_t hi = std::min(n_t, lo + size);
            CSX_CUDA(cudaMemsetAsync(d_count, 0, sizeof(unsigned int), st));
            const uint32_t ts = static_cast<uint32_t>(t);
            if (full) {
                if (pl.fast_delta)
                    tie_collect_kernel<true><<<blocks, 256, 0, st>>>(F, n_items, ts, lo, hi, thr, all, d_hits, d_count, cap);
                else
                    tie_collect_kernel<false><<<blocks, 256, 0, st>>>(F, n_items, ts, lo, hi, thr, all, d_hits, d_count, cap);
            } else {
                if (pl.fast_delta)
                    tie_collect_kernel<true><<<blocks, 256, 0, st>>>(A, n_items, ts, lo, hi, thr, all, d_hits, d_count, cap);
                else
                    tie_collect_kernel<false><<<blocks, 256, 0, st>>>(A, n_items, ts, lo, hi, thr, all, d_hits, d_count, cap);
            }
            CSX_CUDA(cudaGetLastError());
            unsigned int n = 0;
            CSX_CUDA(cudaMemcpyAsync(&n, d_count, sizeof(n), cudaMemcpyDeviceToHost, st));
            CSX_CUDA(cudaStreamSynchronize(st));
            if (n > cap) {  // too many above the root in this chunk: read it in halves
                size = std::max<uint64_t>(1, (hi - lo) / 2);
                continue;
            }
            hits.resize(n);
            if (n) {
                CSX_CUDA(cudaMemcpyAsync(hits.data(), d_hits, n * sizeof(TieHit), cudaMemcpyDeviceToHost, st));
                CSX_CUDA(cudaStreamSynchronize(st));
            }
            std::sort(hits.begin(), hits.end(), [](const TieHit &a, const TieHit &b) { return a.index < b.index; });
            for (const TieHit &x : hits) tie_heap_offer(h, K, x);
            if (h.size() == K) {
                all = false;
                thr = h[0].score;
            }
            lo = hi;
            size *= 2;
        }
    }
    // the reference's order over the replayed heaps and the other survivors
    struct Ranked {
        uint32_t okey;
        uint64_t stream, pos;
        int64_t from_out;  // survivor index, or -1 - (replayed candidate index)
    };
    std::vector<Ranked> all_r;
    std::vector<TieHit> rep_hits;
    std::vector<uint64_t> rep_streams;
    for (uint64_t q = 0; q < cnt; ++q)
        if (!S.count(out[q].stream))
            all_r.push_back({host_okey(out[q].score), out[q].stream, out[q].index, static_cast<int64_t>(q)});
    for (auto &kv : heaps)
        for (size_t i = 0; i < kv.second.size(); ++i) {
            const uint32_t ok = host_okey(kv.second[i].score);
            if (ok < tau) continue;
            all_r.push_back({ok, kv.first, i, -1 - static_cast<int64_t>(rep_hits.size())});
            rep_hits.push_back(kv.second[i]);
            rep_streams.push_back(kv.first);
        }
    if (all_r.size() < cnt) return CSX_ERR_DEVICE_STATE;  // cannot happen: the heaps hold every candidate >= tau
    std::stable_sort(all_r.begin(), all_r.end(), [](const Ranked &a, const Ranked &b) {
        if (a.okey != b.okey) return a.okey > b.okey;
        if (a.stream != b.stream) return a.stream < b.stream;
        return a.pos < b.pos;
    });
    const uint32_t nrep = static_cast<uint32_t>(rep_hits.size());
    std::vector<csx_survivor> regen(nrep);
    if (nrep) {
        CSX_CUDA(cx.tie_streams.ensure(nrep * sizeof(uint64_t)));
        CSX_CUDA(cx.tie_out.ensure(nrep * sizeof(csx_survivor)));
        CSX_CUDA(cudaMemcpyAsync(d_hits, rep_hits.data(), nrep * sizeof(TieHit), cudaMemcpyHostToDevice, st));
        CSX_CUDA(cudaMemcpyAsync(cx.tie_streams.p, rep_streams.data(), nrep * sizeof(uint64_t),
                                 cudaMemcpyHostToDevice, st));
        auto *d_str = static_cast<const uint64_t *>(cx.tie_streams.p);
        auto *d_out = static_cast<csx_survivor *>(cx.tie_out.p);
        const unsigned long long *ids = bufs.ids;
        const unsigned int *tribes = bufs.tribes;
        const int rb = unit_blocks(nrep, 128);
        if (full && pl.fast_delta) tie_regen_full_kernel<true><<<rb, 128, 0, st>>>(F, d_hits, d_str, nrep, ids, tribes, d_out);
        else if (full) tie_regen_full_kernel<false><<<rb, 128, 0, st>>>(F, d_hits, d_str, nrep, ids, tribes, d_out);
        else if (pl.fast_delta) tie_regen_kernel<true><<<rb, 128, 0, st>>>(A, d_hits, d_str, nrep, ids, tribes, d_out);
        else tie_regen_kernel<false><<<rb, 128, 0, st>>>(A, d_hits, d_str, nrep, ids, tribes, d_out);
        CSX_CUDA(cudaGetLastError());
        CSX_CUDA(cudaMemcpyAsync(regen.data(), d_out, nrep * sizeof(csx_survivor), cudaMemcpyDeviceToHost, st));
        CSX_CUDA(cudaStreamSynchronize(st));
        for (uint32_t i = 0; i < nrep; ++i)  // the regenerated score is the replayed one, bit for bit
            if (host_okey(regen[i].score) != host_okey(rep_hits[i].score)) return CSX_ERR_DEVICE_STATE;
    }
    std::vector<csx_survivor> fixed(cnt);
    for (uint64_t q = 0; q < cnt; ++q) {
        const Ranked &r = all_r[q];
        fixed[q] = r.from_out >= 0 ? out[r.from_out] : regen[static_cast<size_t>(-1 - r.from_out)];
    }
    std::copy(fixed.begin(), fixed.end(), out);
    return CSX_OK;
}

// csx_screen / csx_screen_range: host buffers, a private stream, synchronous.
int screen_host(const csx_cfg *cfg, const csx_model *model, const csx_genome *elites, int n_elites,
                uint64_t t_begin, uint64_t t_end, csx_survivor *out, uint64_t out_cap, uint64_t *n_out,
                uint64_t *screened, const csx_model_full *full = nullptr, Shard shard = Shard{}) {
    if (n_out) *n_out = 0;
    if (screened) *screened = 0;
    int rc = check_common(cfg, model, n_elites);
    if (rc) return rc;
    if (!elites || !n_out || (!out && out_cap > 0)) return CSX_ERR_BAD_ARGS;
    if (cfg->lambda == 0) return CSX_OK;
    Context *cx = nullptr;
    rc = current_context(&cx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(cx->mu);
    int dev = 0;
    CSX_CUDA(cudaGetDevice(&dev));
    rc = context_init(*cx, dev);
    if (rc) return rc;
    const uint64_t keep_n = std::min<uint64_t>(cfg->keep, cfg->lambda);
    if (out_cap < keep_n && !(cfg->flags & CSX_FLAG_AS_SHIPPED)) return CSX_ERR_BAD_ARGS;
    CSX_CUDA(cx->genomes.ensure(static_cast<size_t>(n_elites) * sizeof(csx_genome)));
    CSX_CUDA(cx->surv.ensure(static_cast<size_t>(cfg->keep) * sizeof(csx_survivor)));
    CSX_CUDA(cx->result.ensure(4 * sizeof(uint64_t)));
    cudaStream_t st = nullptr;
    CSX_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    auto *dg = static_cast<csx_genome *>(cx->genomes.p);
    auto *ds = static_cast<csx_survivor *>(cx->surv.p);
    auto *dr = static_cast<unsigned long long *>(cx->result.p);
    unsigned long long res[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemcpyAsync(dg, elites, static_cast<size_t>(n_elites) * sizeof(csx_genome),
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        rc = enqueue_screen(*cx, *cfg, *model, dg, n_elites, ds, dr, st, t_begin, t_end, full, shard);
        if (rc == CSX_OK) {
            e = cudaMemcpyAsync(res, dr, sizeof(res), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            const uint64_t cnt = std::min<uint64_t>(res[0], keep_n);
            if (e == cudaSuccess && res[2] == 0 && cnt > 0 && !(cfg->flags & CSX_FLAG_AS_SHIPPED)) {
                e = cudaMemcpyAsync(out, ds, cnt * sizeof(csx_survivor), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                // whole streams only: an item share does not hold a stream's heap
                if (e == cudaSuccess && shard.count == 1 &&
                    !(cfg->flags & (CSX_FLAG_TC_BF16 | CSX_FLAG_TC_FP16)))
                    rc = fix_ties(*cx, *cfg, *model, full, n_elites, t_begin, t_end, out, cnt,
                                  ScreenBufs{static_cast<const float *>(cx->tab.p),
                                             static_cast<const Item *>(cx->items.p), res[3],
                                             static_cast<const unsigned long long *>(cx->ids.p),
                                             static_cast<const unsigned int *>(cx->tribes.p), cx->fin,
                                             cx->fin_kpad},
                                  st);
            }
        }
    }
    cudaStreamDestroy(st);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "csx: %s\n", cudaGetErrorString(e));
        return CSX_ERR_CUDA;
    }
    if (rc) return rc;
    if (res[2] != 0) {
        std::fprintf(stderr, "csx: device error flags 0x%llx\n", res[2]);
        return CSX_ERR_DEVICE_STATE;
    }
    cx->info.items = res[3];
    *n_out = (cfg->flags & CSX_FLAG_AS_SHIPPED) ? 0 : std::min<uint64_t>(res[0], keep_n);
    if (screened) *screened = res[1];
    return CSX_OK;
}

}  // namespace csx

extern "C" {

int csx_screen(const csx_cfg *cfg, const csx_model *model, const csx_genome *elites, int n_elites,
               csx_survivor *out, uint64_t out_cap, uint64_t *n_out, uint64_t *screened) {
    return screen_host(cfg, model, elites, n_elites, 0, 0, out, out_cap, n_out, screened);
}

int csx_screen_full(const csx_cfg *cfg, const csx_model_full *model, const csx_genome *elites, int n_elites,
                    csx_survivor *out, uint64_t out_cap, uint64_t *n_out, uint64_t *screened) {
    if (!model) {
        if (n_out) *n_out = 0;
        if (screened) *screened = 0;
        return CSX_ERR_BAD_ARGS;
    }
    return screen_host(cfg, &kZeroModel, elites, n_elites, 0, 0, out, out_cap, n_out, screened, model);
}

int csx_screen_full_range(const csx_cfg *cfg, const csx_model_full *model, const csx_genome *elites,
                          int n_elites, uint64_t t_begin, uint64_t t_end, csx_survivor *out, uint64_t out_cap,
                          uint64_t *n_out, uint64_t *screened) {
    if (!model || t_end <= t_begin) {
        if (n_out) *n_out = 0;
        if (screened) *screened = 0;
        return CSX_ERR_BAD_ARGS;
    }
    return screen_host(cfg, &kZeroModel, elites, n_elites, t_begin, t_end, out, out_cap, n_out, screened, model);
}

int csx_screen_items(const csx_cfg *cfg, const csx_model *model, const csx_genome *elites, int n_elites,
                     uint32_t shard, uint32_t n_shards, csx_survivor *out, uint64_t out_cap, uint64_t *n_out,
                     uint64_t *screened) {
    if (n_shards == 0 || shard >= n_shards) {
        if (n_out) *n_out = 0;
        if (screened) *screened = 0;
        return CSX_ERR_BAD_ARGS;
    }
    Shard sh;
    sh.index = shard;
    sh.count = n_shards;
    return screen_host(cfg, model, elites, n_elites, 0, 0, out, out_cap, n_out, screened, nullptr, sh);
}

int csx_screen_range(const csx_cfg *cfg, const csx_model *model, const csx_genome *elites, int n_elites,
                     uint64_t t_begin, uint64_t t_end, csx_survivor *out, uint64_t out_cap, uint64_t *n_out,
                     uint64_t *screened) {
    if (t_end <= t_begin) {
        if (n_out) *n_out = 0;
        if (screened) *screened = 0;
        return CSX_ERR_BAD_ARGS;
    }
    return screen_host(cfg, model, elites, n_elites, t_begin, t_end, out, out_cap, n_out, screened);
}

}  // extern "C"

// ---- screen without allocation -----------------------------------------------
//
// csx_screen_device_noalloc: the same pipeline with every piece of device
// scratch carved from one static array compiled into this library, for
// callers that cannot call cudaMalloc: a process whose memory pool owns the
// whole device, or a caller that cannot afford the implicit device-wide
// synchronisation cudaMalloc / cudaFree can bring while its other streams run.
// The array is process-wide, so calls that overlap on the GPU race; the
// control block that must start at zero is cleared on every call.
namespace csx {

constexpr size_t kNoAllocScratchBytes = 32ull << 20;  // held by every GPU that loads the library
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocDevice {
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    int num_sms = 0;
    size_t max_smem = 0;
};
static std::mutex g_noalloc_mu;
static NoAllocDevice g_noalloc[64];

// Once per device, with that device current: the scratch's device address.
// In host code g_noalloc_scratch names a host-side stand-in, never passed on.
// The address is kept for the life of the process: a cudaDeviceReset, which
// unloads this library's device code, is not supported between calls.
int noalloc_setup(int dev, NoAllocDevice **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc[dev];
    if (!d.scratch) {
        void *p = nullptr;
        CSX_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        int v = 0;
        CSX_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
        d.num_sms = v;
        CSX_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        d.max_smem = static_cast<size_t>(v);
        d.scratch = static_cast<unsigned char *>(p);
    }
    *out = &d;
    return CSX_OK;
}

// Plan for the fixed scratch: items of at least 16384 candidates (fewer items
// and checkpoints). A segment's range of cnt candidates holds at most
// ceil(cnt / D) split points, so items <= 2 * segments + lambda / D.
// Checkpoints are sized for one segment's chain (no link margin, where the
// pooled plan adds kLinkSlackCands): a link can land past its segment, and a
// checkpoint the walk cannot store is dropped; split_range then clamps at the
// last stored one, so that segment's last item grows instead (still within
// the items bound above) and the result is unchanged. The pooled plan's margin
// buys smaller items, which this plan does not need.
int plan_noalloc(const NoAllocDevice &dv, const csx_cfg &cfg, const csx_model &model, int ne, Plan *pl) {
    StreamGeom &g = pl->g;
    int src = split_streams(cfg, 0, 0, g);
    if (src) return src;
    const uint64_t my_max = std::max(g.per, g.my_last);
    screen_shape(cfg, model, false, pl);
    pl->smem = screen_smem(pl->sort_n, ne, pl->filter);
    if (pl->smem + 1024 > dv.max_smem) return CSX_ERR_LIMIT;
    int rc = screen_occupancy(screen_fn(pl->fast_delta, pl->filter), dv.num_sms, pl->smem, &pl->grid);
    if (rc) return rc;
    const uint64_t target = 8ull * static_cast<uint64_t>(pl->grid) * kThreads;
    uint64_t d = std::max<uint64_t>(16384, cfg.lambda / target);
    d = std::min<uint64_t>(d, 1ull << 20);
    uint32_t dl = 0;
    while ((2ull << dl) <= d) ++dl;
    g.d_log2 = dl;
    const uint64_t D = 1ull << dl;
    segment_geometry(cfg, kNoAllocSegCands, false, g);
    pl->short_path = my_max <= D;
    pl->items_cap = pl->short_path ? g.nT : 2 * g.n_seg + cfg.lambda / D + 1;
    if (pl->items_cap >= 0xFFFFFFFFull) return CSX_ERR_LIMIT;
    return CSX_OK;
}

// Bump carving of the static scratch (256-byte aligned pieces).
struct Carve {
    unsigned char *base;
    size_t off = 0;
    template <typename T>
    T *take(size_t count) {
        off = (off + 255) & ~static_cast<size_t>(255);
        T *p = reinterpret_cast<T *>(base + off);
        off += count * sizeof(T);
        return p;
    }
};

int enqueue_screen_noalloc(const NoAllocDevice &dv, const csx_cfg &cfg, const csx_model &model,
                           const csx_genome *d_genomes, int ne, csx_survivor *d_out,
                           unsigned long long *d_result, cudaStream_t st) {
    Plan pl;
    int rc = plan_noalloc(dv, cfg, model, ne, &pl);
    if (rc) return rc;
    const StreamGeom &g = pl.g;
    const bool fast = pl.fast_delta;
    const uint32_t nl = static_cast<uint32_t>(pl.grid);
    Carve cv{dv.scratch};
    Ctrl *ctrl = cv.take<Ctrl>(1);
    float *tab = cv.take<float>(static_cast<size_t>(ne + 1) * kNtot);
    auto *ids = cv.take<unsigned long long>(static_cast<size_t>(ne));
    auto *tribes = cv.take<unsigned int>(static_cast<size_t>(ne));
    Item *items = cv.take<Item>(pl.items_cap);
    Entry *lists_a = cv.take<Entry>(static_cast<size_t>(nl) * pl.kpad);
    Entry *lists_b = cv.take<Entry>(static_cast<size_t>((nl + 1) / 2) * pl.kpad);
    SegRec *recs = nullptr;
    uint64_t *ck = nullptr;
    SegOut *so = nullptr;
    uint32_t *off = nullptr;
    if (!pl.short_path) {
        recs = cv.take<SegRec>(g.n_seg);
        ck = cv.take<uint64_t>(g.n_seg * g.ckcap);
        so = cv.take<SegOut>(g.n_seg);
        off = cv.take<uint32_t>(g.n_seg);
    }
    if (cv.off > kNoAllocScratchBytes) {
        std::fprintf(stderr,
                     "csx_screen_device_noalloc: this configuration needs %zu bytes of device scratch; "
                     "the library's static scratch holds %zu\n",
                     cv.off, kNoAllocScratchBytes);
        return CSX_ERR_LIMIT;
    }
    CSX_CUDA(cudaMemsetAsync(ctrl, 0, sizeof(Ctrl), st));
    const SynthConst sc = make_synth(cfg, ne);
    uint32_t launches = 0;
    prep_elites_kernel<<<unit_blocks(static_cast<uint64_t>(ne + 1) * kNtot, 256), 256, 0, st>>>(
        d_genomes, ne, tab, ids, tribes);
    CSX_CUDA(cudaGetLastError());
    rc = enqueue_items(sc, pl, recs, ck, so, off, items, ctrl, st, &launches);
    if (rc) return rc;
    const ScreenArgs A = screen_args(cfg, model, sc, pl, tab, items, ctrl, lists_a);
    screen_fn(fast, pl.filter)<<<pl.grid, kThreads, pl.smem, st>>>(A);
    CSX_CUDA(cudaGetLastError());
    Entry *cur = nullptr;
    rc = enqueue_merge(lists_a, lists_b, nl, pl.kpad, st, &cur, &launches);
    if (rc) return rc;
    if (fast)
        regen_kernel<true><<<unit_blocks(cfg.keep, 128), 128, 0, st>>>(A, cur, ids, tribes, d_out, d_result);
    else
        regen_kernel<false><<<unit_blocks(cfg.keep, 128), 128, 0, st>>>(A, cur, ids, tribes, d_out, d_result);
    CSX_CUDA(cudaGetLastError());
    result_kernel<<<1, 32, 0, st>>>(ctrl, d_result);
    CSX_CUDA(cudaGetLastError());
    return CSX_OK;
}

}  // namespace csx

extern "C" int csx_screen_device_noalloc(const csx_cfg *cfg, const csx_model *model,
                                         const csx_genome *d_elites, int n_elites, csx_survivor *d_out,
                                         uint64_t out_cap, uint64_t *d_result, void *cuda_stream) {
    int rc = check_common(cfg, model, n_elites);
    if (rc) return rc;
    if (cfg->flags & (CSX_FLAG_TC_BF16 | CSX_FLAG_TC_FP16)) return CSX_ERR_BAD_ARGS;  // csx_screen_device only
    if (!d_elites || !d_result || (!d_out && cfg->lambda > 0)) return CSX_ERR_BAD_ARGS;
    if (out_cap < std::min<uint64_t>(cfg->keep, cfg->lambda)) return CSX_ERR_BAD_ARGS;
    int count = 0, dev = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return CSX_ERR_NO_DEVICE;
    }
    CSX_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return CSX_ERR_LIMIT;
    NoAllocDevice *dv = nullptr;
    rc = noalloc_setup(dev, &dv);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    if (cfg->lambda == 0) {
        CSX_CUDA(cudaMemsetAsync(d_result, 0, 4 * sizeof(uint64_t), st));
        return CSX_OK;
    }
    return enqueue_screen_noalloc(*dv, *cfg, *model, d_elites, n_elites, d_out,
                                  reinterpret_cast<unsigned long long *>(d_result), st);
}

#include "csx_batch.cuh"
#include "csx_precision.cuh"

// ---- Model.score of given genomes ---------------------------------------------------
namespace csx {

__global__ void score_genes_kernel(const __grid_constant__ DevModel M, const float *__restrict__ genes, int64_t n,
                                   int ldg, float *__restrict__ out) {
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float g[kNtot];
#pragma unroll
        for (int k = 0; k < kNtot; ++k) g[k] = genes[r * ldg + k];
        out[r] = score_genes_exact(M, g);
    }
}

__global__ void score_full_kernel(const __grid_constant__ FullModel M, const float *__restrict__ genes, int64_t n,
                                  int ldg, float *__restrict__ out) {
    for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < n;
         r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float g[kNtot];
#pragma unroll
        for (int k = 0; k < kNtot; ++k) g[k] = genes[r * ldg + k];
        out[r] = score_full(M, g);
    }
}

}  // namespace csx

extern "C" int csx_score_full(const csx_model_full *model, const float *d_genes, int64_t n, int ldg, float *d_out,
                              void *cuda_stream) {
    if (!model || n < 0 || ldg < kNtot || (n > 0 && (!d_genes || !d_out))) return CSX_ERR_BAD_ARGS;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return CSX_ERR_NO_DEVICE;
    }
    if (n == 0) return CSX_OK;
    int dev = 0, sms = 0;
    CSX_CUDA(cudaGetDevice(&dev));
    CSX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = static_cast<int>(std::min<int64_t>((n + 255) / 256, 16ll * sms));
    score_full_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(cuda_stream)>>>(make_full_model(*model), d_genes, n,
                                                                                  ldg, d_out);
    CSX_CUDA(cudaGetLastError());
    return CSX_OK;
}

extern "C" int csx_score(const csx_model *model, const float *d_genes, int64_t n, int ldg, float *d_out,
                         void *cuda_stream) {
    if (!model || n < 0 || ldg < kNtot || (n > 0 && (!d_genes || !d_out))) return CSX_ERR_BAD_ARGS;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return CSX_ERR_NO_DEVICE;
    }
    if (n == 0) return CSX_OK;
    int dev = 0, sms = 0;
    CSX_CUDA(cudaGetDevice(&dev));
    CSX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = static_cast<int>(std::min<int64_t>((n + 255) / 256, 16ll * sms));
    score_genes_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(cuda_stream)>>>(make_dev_model(*model), d_genes, n,
                                                                                   ldg, d_out);
    CSX_CUDA(cudaGetLastError());
    return CSX_OK;
}
