// csx_batch.cuh — batched islands: many independent screens in one pipeline
// (csx_screen_batch, csx_screen_batch_device). Part of csx_screen.cu's
// translation unit (included there, in order); not a standalone header.
#pragma once

// ---- batched islands -------------------------------------------------------------
//
// Several independent screens in one pipeline. Each island's items are built
// by the single-screen stages on a forked stream of its own (the stages of
// small islands are short of parallel work, so islands overlap). Then either
// form screens them:
//
// * pruned (every island admits the tensor-core pruning bound and clears the
//   pruning floor): each island's pruning screen (csx_prune.cuh) runs over the
//   whole GPU in turn, with its own shared memory and grid, waiting only for
//   its own island's items, and writes its CTA lists into the island's area;
// * otherwise one persistent launch screens every island's items (below): a
//   global counter hands
// out items in island order, a thread whose next item belongs to a later
// island parks it, and when no thread of the CTA has work left on the current
// island the CTA publishes its top-K list for that island and switches to the
// lowest parked island, loading that island's elite table and model into
// shared memory. Counters only grow, so a CTA visits islands in increasing
// order and each at most once; lists of islands it never visits stay zero.
namespace csx {

constexpr int kMaxIslands = CSX_MAX_ISLANDS;

struct IslandDev {
    DevModel m;
    RowModel rm;  // the same coefficients in the screen's consumption order
    SynthConst sc;
    uint64_t seed;
    const float *el;  // (ne + 1) x 29 elite table
    const Item *items;
    Entry *lists_a, *lists_b;  // grid x kpad each (merge ping-pong)
    Ctrl *ctrl;
    const unsigned long long *ids;
    const unsigned int *tribes;
    csx_survivor *out;
    unsigned long long *result;  // 4 words
    uint32_t keep, kpad, ne;
    float err;
    JumpBound jb;
};

struct BatchArgs {
    const IslandDev *isl;
    const unsigned int *base;  // n_islands + 1 prefix sums of the islands' item counts
    unsigned int *next_item;
    uint32_t n_islands, sort_n, ne_max;
};

__global__ void batch_base_kernel(const IslandDev *__restrict__ isl, uint32_t n, unsigned int *__restrict__ base,
                                  unsigned int *__restrict__ next_item) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    unsigned long long s = 0;  // the host keeps the sum of item capacities below 2^32
    for (uint32_t i = 0; i < n; ++i) {
        base[i] = static_cast<unsigned int>(s);
        s += isl[i].ctrl->n_items;
    }
    base[n] = static_cast<unsigned int>(s);
    *next_item = 0;
}

// Island of global item g: the i with b[i] <= g < b[i + 1] (g < b[n]).
__device__ __forceinline__ uint32_t island_of(const unsigned int *b, uint32_t n, unsigned int g) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (b[mid] <= g)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

template <bool kFastDelta>
__device__ __noinline__ float exact_score_isl(const RowModel *m, const SynthConst *sc, const float *el,
                                              uint64_t seed_t, uint64_t p) {
    const CandHead h = cand_head(*sc, seed_t, p);
    return synth_score<kFastDelta, false, true>(*m, *sc, el, seed_t, p, h, nullptr);
}

template <bool kFastDelta, bool kFilter>
__global__ void __launch_bounds__(kThreads, 3) screen_batch_kernel(const __grid_constant__ BatchArgs B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Entry *E = reinterpret_cast<Entry *>(smem_raw);
    float *el = reinterpret_cast<float *>(E + B.sort_n);
    Pend *pend = reinterpret_cast<Pend *>(el + (B.ne_max + 1) * kNtot);  // filter form: exact-order queue
    __shared__ RowModel s_m;
    __shared__ SynthConst s_sc;
    __shared__ unsigned int s_base[kMaxIslands + 1];
    __shared__ const Item *s_items;
    __shared__ Ctrl *s_ctrl;
    __shared__ Entry *s_lists;
    __shared__ unsigned long long s_seed, s_t1, s_t2;
    __shared__ unsigned int s_buf_n, s_pend_n, s_next, s_keep, s_kpad, s_buf_cap;
    __shared__ int s_cur;
    __shared__ float s_ts, s_err;
    __shared__ JumpBound s_jb;

    const uint32_t tid = threadIdx.x;
    for (uint32_t i = tid; i <= B.n_islands; i += kThreads) s_base[i] = B.base[i];
    if (tid == 0) {
        s_cur = -1;
        s_buf_n = 0;
        s_pend_n = 0;
        s_kpad = 0;
        s_keep = 0;
        s_buf_cap = 0;
    }
    __syncthreads();
    const unsigned int total = s_base[B.n_islands];

    // item: the global index while parked, the island-local index while valid
    unsigned int item = atomicAdd(B.next_item, 1u);
    bool parked = item < total;  // holds an item of an island the CTA has not reached
    bool valid = false;          // working on an item of the current island
    uint64_t seed_t = 0, p = 0;
    uint32_t left = 0, dcand = 0, ddraw = 0;
    unsigned long long screened = 0, exact = 0;
    unsigned int gk = 0;
    uint32_t round = 0;
    // a held entry: the buffer was full (exact-all form) or the queue was (filter form)
    bool has_def = false;
    Entry def{0ull, 0ull};
    Pend pdef{0u, 0u, 0u};

    // merge the buffer into the CTA's sorted list; publishes the island's threshold
    auto merge = [&]() {
        cta_sort_desc(E, B.sort_n);
        for (uint32_t i = s_kpad + tid; i < B.sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
        if (tid == 0) {
            s_buf_n = 0;
            const Entry kth = E[s_keep - 1];
            if (kth.k1 != 0ull) {
                s_t1 = kth.k1;
                s_t2 = kth.k2;
                const unsigned int ok = static_cast<unsigned int>(kth.k1 >> 32);
                s_ts = okey_score(ok);
                atomicMax(&s_ctrl->gtau, ok);
            }
        }
        __syncthreads();
    };
    // reference-order score of a queued candidate; enters the buffer if it beats the threshold
    auto rescore = [&](const Pend &q, unsigned long long t1, unsigned long long t2, float ts) {
        const Item it = s_items[q.item];
        const float s =
            exact_score_isl<kFastDelta>(&s_m, &s_sc, el, stream_seed(s_seed, it.stream), it.draw0 + q.ddraw);
        ++exact;
        if (s >= ts) {
            const unsigned long long k1 =
                (static_cast<unsigned long long>(score_okey(s)) << 32) | static_cast<unsigned int>(~q.item);
            const unsigned long long k2 = (static_cast<unsigned long long>(~q.dcand) << 32) | q.ddraw;
            E[s_kpad + atomicAdd(&s_buf_n, 1u)] = Entry{k1, k2};  // score >= ts: ties with the K-th kept
        }
    };

    for (;;) {
        __syncthreads();
        const unsigned int pn = min(s_pend_n, kPendCap);
        const int any = __syncthreads_or(valid || has_def);
        const int any_def = __syncthreads_or(has_def);
        const int cur = s_cur;
        if (kFilter && cur >= 0 && (pn >= kThreads || any_def || (!any && pn > 0))) {
            // a flush appends <= pn + 256 <= 768 entries
            if (s_buf_n + kPendCap + kThreads > s_buf_cap) merge();
            unsigned long long t1 = s_t1, t2 = s_t2;
            float ts = s_ts;
            const unsigned int g = *reinterpret_cast<volatile unsigned int *>(&s_ctrl->gtau);
            if ((static_cast<unsigned long long>(g) << 32) > t1) {
                t1 = static_cast<unsigned long long>(g) << 32;
                t2 = 0;
                ts = okey_score(g);
            }
            for (uint32_t i = tid; i < pn; i += kThreads) rescore(pend[i], t1, t2, ts);
            if (has_def) {
                rescore(pdef, t1, t2, ts);
                has_def = false;
            }
            __syncthreads();
            if (tid == 0) s_pend_n = 0;
            __syncthreads();
        }
        const unsigned int bn = s_buf_n;
        if (cur >= 0 && (bn >= s_buf_cap / 2 || (!any && bn > 0))) merge();
        if (!any) {
            if (cur >= 0) {  // publish this CTA's list and counts for the island it leaves
                Entry *out = s_lists + static_cast<size_t>(blockIdx.x) * s_kpad;
                for (uint32_t i = tid; i < s_kpad; i += kThreads) out[i] = E[i];
                for (int o = 16; o > 0; o >>= 1) {
                    screened += __shfl_down_sync(0xffffffffu, screened, o);
                    exact += __shfl_down_sync(0xffffffffu, exact, o);
                }
                if ((tid & 31) == 0) {
                    atomicAdd(&s_ctrl->screened, screened);
                    if (kFilter) atomicAdd(&s_ctrl->exact_evals, exact);
                }
                screened = 0;
                exact = 0;
            }
            if (tid == 0) s_next = 0xFFFFFFFFu;
            __syncthreads();
            if (parked) atomicMin(&s_next, island_of(s_base, B.n_islands, item));
            __syncthreads();
            const unsigned int nx = s_next;
            if (nx == 0xFFFFFFFFu) break;
            const IslandDev *I = B.isl + nx;
            const uint32_t *src = reinterpret_cast<const uint32_t *>(&I->rm);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&s_m);
            for (uint32_t i = tid; i < sizeof(RowModel) / 4; i += kThreads) dst[i] = src[i];
            const uint32_t ne = I->ne;
            for (uint32_t i = tid; i < (ne + 1) * kNtot; i += kThreads) el[i] = I->el[i];
            for (uint32_t i = tid; i < B.sort_n; i += kThreads) E[i] = Entry{0ull, 0ull};
            if (tid == 0) {
                s_sc = I->sc;
                s_seed = I->seed;
                s_items = I->items;
                s_ctrl = I->ctrl;
                s_lists = I->lists_a;
                s_keep = I->keep;
                s_kpad = I->kpad;
                s_buf_cap = B.sort_n - I->kpad;
                s_err = I->err;
                s_jb = I->jb;
                s_cur = static_cast<int>(nx);
                s_buf_n = 0;
                s_t1 = 0;
                s_t2 = 0;
                s_ts = -INFINITY;
            }
            __syncthreads();
            gk = 0;
            round = 0;
            if (parked && item >= s_base[nx] && item < s_base[nx + 1]) {
                parked = false;
                item -= s_base[nx];
                const Item it = s_items[item];
                seed_t = stream_seed(s_seed, it.stream);
                p = it.draw0;
                left = it.n;
                dcand = 0;
                ddraw = 0;
                valid = left > 0;
            }
            continue;
        }
        const uint32_t kp = s_kpad, bcap = s_buf_cap;
        Entry *buf = E + kp;
        if (!kFilter && has_def) {  // the merge above emptied the buffer: room for every held entry
            const unsigned int slot = atomicAdd(&s_buf_n, 1u);
            buf[slot] = def;
            has_def = false;
        }
        unsigned long long t1 = s_t1, t2 = s_t2;
        float ts = s_ts;
        if ((round++ & 7u) == 0) gk = *reinterpret_cast<volatile unsigned int *>(&s_ctrl->gtau);
        if ((static_cast<unsigned long long>(gk) << 32) > t1) {
            t1 = static_cast<unsigned long long>(gk) << 32;
            t2 = 0;
            ts = okey_score(gk);
        }
        const float tlo = kFilter ? __fsub_rd(ts, s_err) : ts;
#pragma unroll 1
        for (int r = 0; r < kRounds && valid && !has_def; ++r) {
            // The model lives in shared memory here: keep its loads inside the
            // loop (hoisted, 166 coefficients would not fit in registers).
            asm volatile("" ::: "memory");
            const CandHead h = cand_head(s_sc, seed_t, p);
            float s;
            if (kFilter) {  // to the queue; scored in the reference order at the next flush
                s = synth_score<kFastDelta, false, false>(s_m, s_sc, el, seed_t, p, h, nullptr);
                if (s >= __fsub_rd(tlo, s_jb.c[h.jidx])) {
                    const unsigned int slot = atomicAdd(&s_pend_n, 1u);
                    if (slot < kPendCap) {
                        pend[slot] = Pend{item, dcand, ddraw};
                    } else {
                        has_def = true;
                        pdef = Pend{item, dcand, ddraw};
                    }
                }
                s = -INFINITY;
            } else {
                s = synth_score<kFastDelta, false>(s_m, s_sc, el, seed_t, p, h, nullptr);
            }
            if (!kFilter && s >= ts) {  // ties with the running K-th score enter too
                const unsigned long long k1 =
                    (static_cast<unsigned long long>(score_okey(s)) << 32) | static_cast<unsigned int>(~item);
                const unsigned long long k2 = (static_cast<unsigned long long>(~dcand) << 32) | ddraw;
                const unsigned int slot = atomicAdd(&s_buf_n, 1u);
                if (slot < bcap) {
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
                valid = false;
                item = atomicAdd(B.next_item, 1u);
                if (item < total) {
                    const unsigned int lo = s_base[cur], hi = s_base[cur + 1];
                    if (item >= lo && item < hi) {
                        item -= lo;
                        const Item it = s_items[item];
                        seed_t = stream_seed(s_seed, it.stream);
                        p = it.draw0;
                        left = it.n;
                        dcand = 0;
                        ddraw = 0;
                        valid = left > 0;
                    } else {
                        parked = true;
                    }
                }
            }
        }
    }
}

__global__ void merge_batch_kernel(const IslandDev *__restrict__ isl, uint32_t nl, int b_to_a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const IslandDev &I = isl[blockIdx.y];
    merge_pair(b_to_a ? I.lists_b : I.lists_a, nl, b_to_a ? I.lists_a : I.lists_b, I.kpad, blockIdx.x,
               reinterpret_cast<Entry *>(smem_raw));
}

template <bool kFastDelta>
__global__ void regen_batch_kernel(const IslandDev *__restrict__ isl, int final_in_b) {
    const IslandDev &I = isl[blockIdx.y];
    regen_one<kFastDelta>(I.m, I.sc, I.seed, I.el, I.items, I.ctrl, final_in_b ? I.lists_b : I.lists_a, I.keep,
                          I.ids, I.tribes, I.out, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void batch_result_kernel(const IslandDev *__restrict__ isl, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Ctrl *c = isl[i].ctrl;
    unsigned long long *r = isl[i].result;
    r[0] = c->n_out;
    r[1] = c->screened;
    r[2] = c->err;
    r[3] = c->n_items;
}

using BatchFn = void (*)(BatchArgs);

BatchFn batch_fn(bool fast_delta, bool filter) {
    if (fast_delta) return filter ? screen_batch_kernel<true, true> : screen_batch_kernel<true, false>;
    return filter ? screen_batch_kernel<false, true> : screen_batch_kernel<false, false>;
}


RowModel make_row_model(const DevModel &m) {
    RowModel r{};
    for (int k = 0; k < 16; ++k) {
        for (int l = 0; l <= k; ++l) r.v[row_off(k) + l] = m.wq[tri(k, l)];
        r.v[row_off(k) + k + 1] = m.wlin[k];
    }
    for (int k = 16; k < kNtot; ++k) r.v[kRowLin16 + k - 16] = m.wlin[k];
    r.v[kRowW16] = m.w16;
    r.v[kRowW16 + 1] = m.w0;
    r.v[kRowW16 + 2] = m.tail ? 1.0f : 0.0f;
    return r;
}


struct IslandBufs {
    const csx_genome *genomes = nullptr;
    float *tab = nullptr;
    unsigned long long *ids = nullptr;
    unsigned int *tribes = nullptr;
    Ctrl *ctrl = nullptr;
    Item *items = nullptr;
    Entry *la = nullptr, *lb = nullptr;
    SegRec *recs = nullptr;
    uint64_t *ck = nullptr;
    SegOut *so = nullptr;
    uint32_t *off = nullptr;
};

struct BatchLayout {
    int n = 0;
    std::vector<Plan> pl;
    std::vector<csx_cfg> cfg;
    std::vector<int> ne;
    std::vector<IslandBufs> b;
    bool fast = true, filter = true;
    uint32_t sort_n = 0, kpad_max = 0, keep_max = 0, ne_max = 0;
    size_t smem = 0;
    int grid = 0;
    IslandDev *d_isl = nullptr;
    unsigned int *d_base = nullptr, *d_next = nullptr;
    Ctrl *ctrl_all = nullptr;
    Entry *lists_all = nullptr;
    size_t lists_bytes = 0;
    // the pruned batch: every island's pruning screen (csx_prune.cuh) in turn
    bool prune = false;
    std::vector<PruneArgs> pargs;
    uint32_t *pub = nullptr;  // kPruneMs x grid, cleared before each island
};

int batch_context_init(Context &cx) {
    if (!cx.pinned) CSX_CUDA(cudaMallocHost(&cx.pinned, kMaxIslands * sizeof(IslandDev)));
    if (!cx.desc_ev) CSX_CUDA(cudaEventCreateWithFlags(&cx.desc_ev, cudaEventDisableTiming));
    if (!cx.ev_fork) CSX_CUDA(cudaEventCreateWithFlags(&cx.ev_fork, cudaEventDisableTiming));
    for (int i = 0; i < kMaxIslands; ++i) {
        if (!cx.aux[i]) CSX_CUDA(cudaStreamCreateWithFlags(&cx.aux[i], cudaStreamNonBlocking));
        if (!cx.ev_join[i]) CSX_CUDA(cudaEventCreateWithFlags(&cx.ev_join[i], cudaEventDisableTiming));
    }
    if (!cx.pst) CSX_CUDA(cudaStreamCreateWithFlags(&cx.pst, cudaStreamNonBlocking));
    return CSX_OK;
}

// Plans, shared-memory shape, grid and device buffers of a batch; writes the
// island descriptors to the page-locked staging area. No stream work.
int batch_prepare(Context &cx, int n, const csx_cfg *cfgs, const csx_model *models, const int *n_elites,
                  const csx_genome *d_genomes, const csx_batch_tune *tune, csx_survivor *d_out,
                  unsigned long long *d_result, BatchLayout *L) {
    L->n = n;
    L->pl.assign(n, Plan{});
    L->cfg.assign(cfgs, cfgs + n);
    L->ne.assign(n_elites, n_elites + n);
    L->b.assign(n, IslandBufs{});
    int ne_max = 0;
    for (int i = 0; i < n; ++i) {
        const csx_cfg &c = cfgs[i];
        const bool fast = std::isfinite(c.sigma) && std::fabs(c.sigma) <= 1.0e38f &&
                          (c.sigma == 0.0f || std::fabs(c.sigma) >= 1.0e-30f);
        L->fast = L->fast && fast;
        L->filter = L->filter && !(c.flags & CSX_FLAG_EXACT_ALL) && filter_bound(models[i]) > 0.0f;
        const uint32_t kpad = list_kpad(c.keep);
        L->kpad_max = std::max(L->kpad_max, kpad);
        L->keep_max = std::max<uint32_t>(L->keep_max, static_cast<uint32_t>(c.keep));
        L->sort_n = std::max(L->sort_n, pow2_at_least(kpad + 4ull * kThreads));
        ne_max = std::max(ne_max, n_elites[i]);
    }
    L->ne_max = static_cast<uint32_t>(ne_max);

    // plans (the grid is set below; item and segment sizes do not depend on it)
    uint64_t items_sum = 0;
    L->prune = true;
    for (int i = 0; i < n; ++i) {
        if (cfgs[i].lambda == 0) continue;
        int rc = make_plan(cx, cfgs[i], models[i], n_elites[i], &L->pl[i], 1, tune ? tune->item_cands : 0,
                           tune ? tune->seg_cands : 0);
        if (rc) return rc;
        items_sum += L->pl[i].items_cap;
        L->prune = L->prune && L->pl[i].prune_ok && L->pl[i].prune_tc;
    }
    if (items_sum >= 0xFFFFFFFFull) return CSX_ERR_LIMIT;

    int per_sm = 0;
    const int cap = tune && tune->ctas_per_sm > 0 ? static_cast<int>(tune->ctas_per_sm) : 3;
    if (L->prune) {
        // every island's pruning screen with the tensor-core bound, one after
        // another, each with its own shared memory and up to three CTAs per SM
        // (as the single screen); the lists are laid out for the widest grid
        L->smem = 0;
        for (int i = 0; i < n; ++i) {
            if (cfgs[i].lambda == 0) continue;
            Plan &pl = L->pl[i];
            pl.el_smem = prune_el_smem(pl.sort_n, n_elites[i], pl.nb, cx.num_sms, true, cx.max_smem);
            pl.smem = prune_smem(pl.sort_n, n_elites[i], pl.nb, cx.num_sms, true, pl.el_smem);
            if (pl.smem + 1024 > cx.max_smem) return CSX_ERR_LIMIT;
            const int fit = std::min(cap, std::max(1, static_cast<int>((228u << 10) / (pl.smem + 1024))));
            pl.grid = fit * cx.num_sms;
            L->smem = std::max(L->smem, pl.smem);
            per_sm = std::max(per_sm, fit);
        }
        per_sm = std::max(per_sm, 1);
        for (int nb : {16, kNtot})
            CSX_CUDA(cudaFuncSetAttribute(screen_p_fn(nb, true, true, false),
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(L->smem)));
    } else {
        L->smem = screen_smem(L->sort_n, ne_max, L->filter);
        if (L->smem + 2048 > cx.max_smem) return CSX_ERR_LIMIT;
        BatchFn fn = batch_fn(L->fast, L->filter);
        CSX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(L->smem)));
        CSX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, L->smem));
        per_sm = std::max(1, per_sm);
    }
    if (tune && tune->ctas_per_sm > 0) per_sm = std::min(per_sm, cap);
    L->grid = per_sm * cx.num_sms;
    if (!L->prune)
        for (int i = 0; i < n; ++i) L->pl[i].grid = L->grid;
    const size_t msmem = 2ull * L->kpad_max * sizeof(Entry);
    CSX_CUDA(cudaFuncSetAttribute(merge_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(msmem)));

    // carve: a sizing pass, then the real one
    const uint32_t nl = static_cast<uint32_t>(L->grid);
    auto carve = [&](unsigned char *base) -> size_t {
        Carve cv{base};
        L->d_isl = cv.take<IslandDev>(n);
        L->d_base = cv.take<unsigned int>(n + 1);
        L->d_next = cv.take<unsigned int>(1);
        L->ctrl_all = cv.take<Ctrl>(n);
        L->pub = L->prune ? cv.take<uint32_t>(static_cast<size_t>(kPruneMs) * nl) : nullptr;
        const size_t lists0 = (cv.off + 255) & ~static_cast<size_t>(255);
        for (int i = 0; i < n; ++i) {
            const uint32_t kpad = list_kpad(cfgs[i].keep);
            L->b[i].la = cv.take<Entry>(static_cast<size_t>(nl) * kpad);
        }
        L->lists_all = reinterpret_cast<Entry *>(base + lists0);
        L->lists_bytes = cv.off - lists0;
        for (int i = 0; i < n; ++i) {
            IslandBufs &b = L->b[i];
            const Plan &pl = L->pl[i];
            const uint32_t kpad = list_kpad(cfgs[i].keep);
            b.ctrl = L->ctrl_all + i;
            b.lb = cv.take<Entry>(static_cast<size_t>((nl + 1) / 2) * kpad);
            b.tab = cv.take<float>(static_cast<size_t>(n_elites[i] + 1) * kNtot);
            b.ids = cv.take<unsigned long long>(static_cast<size_t>(n_elites[i]));
            b.tribes = cv.take<unsigned int>(static_cast<size_t>(n_elites[i]));
            if (cfgs[i].lambda == 0) continue;
            b.items = cv.take<Item>(pl.items_cap);
            if (!pl.short_path) {
                b.recs = cv.take<SegRec>(pl.g.n_seg);
                b.ck = cv.take<uint64_t>(pl.g.n_seg * pl.g.ckcap);
                b.so = cv.take<SegOut>(pl.g.n_seg);
                b.off = cv.take<uint32_t>(pl.g.n_seg);
            }
        }
        return cv.off;
    };
    const size_t bytes = carve(nullptr);
    CSX_CUDA(cx.batch.ensure(bytes));
    carve(static_cast<unsigned char *>(cx.batch.p));

    // descriptors (the previous call's copy must have left the staging area)
    if (cx.desc_pending) {
        CSX_CUDA(cudaEventSynchronize(cx.desc_ev));
        cx.desc_pending = false;
    }
    auto *hd = static_cast<IslandDev *>(cx.pinned);
    const csx_genome *g = d_genomes;
    uint64_t out_off = 0;
    for (int i = 0; i < n; ++i) {
        IslandBufs &b = L->b[i];
        b.genomes = g;
        g += n_elites[i];
        IslandDev &d = hd[i];
        d.m = make_dev_model(models[i]);
        d.rm = make_row_model(d.m);
        d.sc = make_synth(cfgs[i], n_elites[i]);
        d.seed = cfgs[i].seed;
        d.el = b.tab;
        d.items = b.items;
        d.lists_a = b.la;
        d.lists_b = b.lb;
        d.ctrl = b.ctrl;
        d.ids = b.ids;
        d.tribes = b.tribes;
        d.out = d_out + out_off;
        d.result = d_result + 4 * i;
        d.keep = static_cast<uint32_t>(cfgs[i].keep);
        d.kpad = list_kpad(cfgs[i].keep);
        d.ne = static_cast<uint32_t>(n_elites[i]);
        d.err = filter_bound(models[i]);
        jump_bound(models[i], &d.jb);
        out_off += cfgs[i].keep;
    }
    L->pargs.assign(n, PruneArgs{});
    if (L->prune) {
        for (int i = 0; i < n; ++i) {
            if (cfgs[i].lambda == 0) continue;
            const Plan &pl = L->pl[i];
            const IslandBufs &b = L->b[i];
            PruneArgs &P = L->pargs[i];
            static_cast<ScreenArgs &>(P) = screen_args(cfgs[i], models[i], make_synth(cfgs[i], n_elites[i]), pl,
                                                       b.tab, b.items, b.ctrl, b.la);
            P.pc = pl.pc;
            P.tc = pl.ptc;
            P.pub = L->pub;
            P.sel_cap = 8u * static_cast<uint32_t>(cx.num_sms);
            P.el_smem = pl.el_smem ? 1u : 0u;
        }
    }
    return CSX_OK;
}

// Stream work of a prepared batch on `st` (capturable: no allocation, no
// synchronisation). Returns the number of kernels enqueued in *launches.
int batch_enqueue(Context &cx, const BatchLayout &L, cudaStream_t st, bool capturing, uint32_t *launches) {
    const int n = L.n;
    uint32_t nk = 0;
    CSX_CUDA(cudaMemcpyAsync(L.d_isl, cx.pinned, n * sizeof(IslandDev), cudaMemcpyHostToDevice, st));
    if (!capturing) {
        CSX_CUDA(cudaEventRecord(cx.desc_ev, st));
        cx.desc_pending = true;
    }
    CSX_CUDA(cudaMemsetAsync(L.ctrl_all, 0, n * sizeof(Ctrl), st));
    CSX_CUDA(cudaMemsetAsync(L.lists_all, 0, L.lists_bytes, st));
    CSX_CUDA(cudaEventRecord(cx.ev_fork, st));
    for (int i = 0; i < n; ++i) {
        cudaStream_t a = cx.aux[i];
        const IslandBufs &b = L.b[i];
        const Plan &pl = L.pl[i];
        const StreamGeom &g = pl.g;
        const int ne = L.ne[i];
        CSX_CUDA(cudaStreamWaitEvent(a, cx.ev_fork, 0));
        prep_elites_kernel<<<unit_blocks(static_cast<uint64_t>(ne + 1) * kNtot, 256), 256, 0, a>>>(
            b.genomes, ne, b.tab, b.ids, b.tribes);
        CSX_CUDA(cudaGetLastError());
        ++nk;
        if (L.cfg[i].lambda > 0) {
            const SynthConst sc = make_synth(L.cfg[i], ne);
            const int rc = enqueue_items(sc, pl, b.recs, b.ck, b.so, b.off, b.items, b.ctrl, a, &nk);
            if (rc) return rc;
        }
        CSX_CUDA(cudaEventRecord(cx.ev_join[i], a));
        if (!L.prune) CSX_CUDA(cudaStreamWaitEvent(st, cx.ev_join[i], 0));
    }
    if (L.prune) {
        // island i's screen waits only for island i's items: the later
        // islands' item building overlaps the earlier screens
        for (int i = 0; i < n; ++i) {
            CSX_CUDA(cudaStreamWaitEvent(st, cx.ev_join[i], 0));
            if (L.cfg[i].lambda == 0) continue;
            const Plan &pl = L.pl[i];
            CSX_CUDA(cudaMemsetAsync(L.pub, 0, static_cast<size_t>(kPruneMs) * pl.grid * sizeof(uint32_t), st));
            screen_p_fn(pl.nb, true, true, false)<<<pl.grid, kThreads, pl.smem, st>>>(L.pargs[i]);
            CSX_CUDA(cudaGetLastError());
            ++nk;
        }
    } else {
        batch_base_kernel<<<1, 32, 0, st>>>(L.d_isl, static_cast<uint32_t>(n), L.d_base, L.d_next);
        CSX_CUDA(cudaGetLastError());
        BatchArgs B;
        B.isl = L.d_isl;
        B.base = L.d_base;
        B.next_item = L.d_next;
        B.n_islands = static_cast<uint32_t>(n);
        B.sort_n = L.sort_n;
        B.ne_max = L.ne_max;
        batch_fn(L.fast, L.filter)<<<L.grid, kThreads, L.smem, st>>>(B);
        CSX_CUDA(cudaGetLastError());
        nk += 2;
    }
    const size_t msmem = 2ull * L.kpad_max * sizeof(Entry);
    uint32_t nl = static_cast<uint32_t>(L.grid);
    int in_b = 0;
    while (nl > 1) {
        const uint32_t m = (nl + 1) / 2;
        merge_batch_kernel<<<dim3(m, n), 256, msmem, st>>>(L.d_isl, nl, in_b);
        CSX_CUDA(cudaGetLastError());
        ++nk;
        in_b ^= 1;
        nl = m;
    }
    const dim3 rg(unit_blocks(std::max<uint32_t>(1, L.keep_max), 128), n);
    if (L.fast)
        regen_batch_kernel<true><<<rg, 128, 0, st>>>(L.d_isl, in_b);
    else
        regen_batch_kernel<false><<<rg, 128, 0, st>>>(L.d_isl, in_b);
    CSX_CUDA(cudaGetLastError());
    batch_result_kernel<<<unit_blocks(n, 64), 64, 0, st>>>(L.d_isl, static_cast<uint32_t>(n));
    CSX_CUDA(cudaGetLastError());
    nk += 2;
    *launches = nk;
    return CSX_OK;
}

int check_batch(int n, const csx_cfg *cfgs, const csx_model *models, const int *n_elites) {
    if (n < 1 || n > kMaxIslands || !cfgs || !models || !n_elites) return n > kMaxIslands ? CSX_ERR_LIMIT
                                                                                        : CSX_ERR_BAD_ARGS;
    for (int i = 0; i < n; ++i) {
        int rc = check_common(&cfgs[i], &models[i], n_elites[i]);
        if (rc) return rc;
        if (cfgs[i].flags & (CSX_FLAG_TC_BF16 | CSX_FLAG_TC_FP16)) return CSX_ERR_BAD_ARGS;  // single screens only
    }
    return CSX_OK;
}

}  // namespace csx

extern "C" {

int csx_screen_batch_device(int n_islands, const csx_cfg *cfgs, const csx_model *models,
                            const csx_genome *d_elites, const int *n_elites, const csx_batch_tune *tune,
                            csx_survivor *d_out, uint64_t *d_result, void *cuda_stream) {
    int rc = check_batch(n_islands, cfgs, models, n_elites);
    if (rc) return rc;
    if (!d_elites || !d_out || !d_result) return CSX_ERR_BAD_ARGS;
    Context *cx = nullptr;
    rc = current_context(&cx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(cx->mu);
    int dev = 0;
    CSX_CUDA(cudaGetDevice(&dev));
    if ((rc = context_init(*cx, dev)) || (rc = batch_context_init(*cx))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CSX_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) return CSX_ERR_BAD_ARGS;  // csx_screen_batch captures its own graph
    BatchLayout L;
    rc = batch_prepare(*cx, n_islands, cfgs, models, n_elites, d_elites, tune, d_out,
                       reinterpret_cast<unsigned long long *>(d_result), &L);
    if (rc) return rc;
    CSX_CUDA(cudaStreamWaitEvent(st, cx->done, 0));
    uint32_t launches = 0;
    rc = batch_enqueue(*cx, L, st, false, &launches);
    if (rc) return rc;
    CSX_CUDA(cudaEventRecord(cx->done, st));
    cx->binfo = csx_batch_info{};
    cx->binfo.islands = static_cast<uint32_t>(n_islands);
    cx->binfo.launches = launches;
    cx->binfo.screen_ctas = static_cast<uint32_t>(L.grid);
    return CSX_OK;
}

int csx_screen_batch(int n_islands, const csx_cfg *cfgs, const csx_model *models, const csx_genome *elites,
                     const int *n_elites, const csx_batch_tune *tune, csx_survivor *out, uint64_t *n_out,
                     uint64_t *screened) {
    int rc = check_batch(n_islands, cfgs, models, n_elites);
    if (rc) return rc;
    if (!elites || !out || !n_out) return CSX_ERR_BAD_ARGS;
    Context *cx = nullptr;
    rc = current_context(&cx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(cx->mu);
    int dev = 0;
    CSX_CUDA(cudaGetDevice(&dev));
    if ((rc = context_init(*cx, dev)) || (rc = batch_context_init(*cx))) return rc;
    uint64_t ne_sum = 0, keep_sum = 0;
    for (int i = 0; i < n_islands; ++i) {
        ne_sum += static_cast<uint64_t>(n_elites[i]);
        keep_sum += cfgs[i].keep;
    }
    CSX_CUDA(cx->b_genomes.ensure(ne_sum * sizeof(csx_genome)));
    CSX_CUDA(cx->b_surv.ensure(keep_sum * sizeof(csx_survivor)));
    CSX_CUDA(cx->b_result.ensure(4ull * n_islands * sizeof(uint64_t)));
    auto *dg = static_cast<csx_genome *>(cx->b_genomes.p);
    auto *ds = static_cast<csx_survivor *>(cx->b_surv.p);
    auto *dr = static_cast<unsigned long long *>(cx->b_result.p);
    BatchLayout L;
    rc = batch_prepare(*cx, n_islands, cfgs, models, n_elites, dg, tune, ds, dr, &L);
    if (rc) return rc;
    cudaStream_t st = cx->pst;
    CSX_CUDA(cudaStreamWaitEvent(st, cx->done, 0));
    CSX_CUDA(cudaMemcpyAsync(dg, elites, ne_sum * sizeof(csx_genome), cudaMemcpyHostToDevice, st));

    const auto t0 = std::chrono::steady_clock::now();
    CSX_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    uint32_t launches = 0;
    rc = batch_enqueue(*cx, L, st, true, &launches);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (rc || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (ce != cudaSuccess) std::fprintf(stderr, "csx: stream capture failed: %s\n", cudaGetErrorString(ce));
        return rc ? rc : CSX_ERR_CUDA;
    }
    if (cx->gexec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(cx->gexec, graph, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(cx->gexec);
            cx->gexec = nullptr;
        }
    }
    if (!cx->gexec) {
        const cudaError_t ie = cudaGraphInstantiate(&cx->gexec, graph, 0);
        if (ie != cudaSuccess) {
            cudaGraphDestroy(graph);
            cx->gexec = nullptr;
            std::fprintf(stderr, "csx: graph instantiate failed: %s\n", cudaGetErrorString(ie));
            return CSX_ERR_CUDA;
        }
    }
    size_t nodes = 0;
    cudaGraphGetNodes(graph, nullptr, &nodes);
    cudaGraphDestroy(graph);
    const auto t1 = std::chrono::steady_clock::now();

    CSX_CUDA(cudaEventRecord(cx->ev[0], st));
    CSX_CUDA(cudaGraphLaunch(cx->gexec, st));
    CSX_CUDA(cudaEventRecord(cx->ev[1], st));
    std::vector<unsigned long long> res(4ull * n_islands);
    CSX_CUDA(cudaMemcpyAsync(res.data(), dr, res.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    CSX_CUDA(cudaStreamSynchronize(st));
    uint64_t off = 0;
    bool bad = false;
    for (int i = 0; i < n_islands; ++i) {
        const uint64_t keep_n = std::min<uint64_t>(cfgs[i].keep, cfgs[i].lambda);
        const uint64_t cnt = std::min<uint64_t>(res[4 * i], keep_n);
        bad = bad || res[4 * i + 2] != 0;
        n_out[i] = (cfgs[i].flags & CSX_FLAG_AS_SHIPPED) ? 0 : cnt;
        if (screened) screened[i] = res[4 * i + 1];
        if (cnt > 0 && res[4 * i + 2] == 0)
            CSX_CUDA(cudaMemcpyAsync(out + off, ds + off, cnt * sizeof(csx_survivor), cudaMemcpyDeviceToHost, st));
        off += cfgs[i].keep;
    }
    CSX_CUDA(cudaStreamSynchronize(st));
    // exact ties as the reference's per-stream heaps order them (fix_ties);
    // the merge tree leaves each island's final list in lists_b after an odd
    // number of levels
    bool in_b = false;
    for (uint32_t nl = static_cast<uint32_t>(L.grid); nl > 1; nl = (nl + 1) / 2) in_b = !in_b;
    off = 0;
    for (int i = 0; i < n_islands && !bad; ++i) {
        const uint64_t cnt = std::min<uint64_t>(res[4 * i], std::min<uint64_t>(cfgs[i].keep, cfgs[i].lambda));
        if (cnt > 0 && !(cfgs[i].flags & CSX_FLAG_AS_SHIPPED)) {
            const IslandBufs &b = L.b[i];
            rc = fix_ties(*cx, cfgs[i], models[i], nullptr, n_elites[i], 0, 0, out + off, cnt,
                          ScreenBufs{b.tab, b.items, res[4 * i + 3], b.ids, b.tribes, in_b ? b.lb : b.la,
                                     L.pl[i].kpad},
                          st);
            if (rc) return rc;
        }
        off += cfgs[i].keep;
    }
    CSX_CUDA(cudaEventRecord(cx->done, st));
    cx->binfo = csx_batch_info{};
    cx->binfo.islands = static_cast<uint32_t>(n_islands);
    cx->binfo.launches = launches;
    cx->binfo.screen_ctas = static_cast<uint32_t>(L.grid);
    cx->binfo.graph_nodes = static_cast<uint32_t>(nodes);
    cx->binfo.ms_capture = std::chrono::duration<float, std::milli>(t1 - t0).count();
    CSX_CUDA(cudaEventElapsedTime(&cx->binfo.ms_device, cx->ev[0], cx->ev[1]));
    if (bad) {
        std::fprintf(stderr, "csx: device error flags in a batch island\n");
        for (int i = 0; i < n_islands; ++i) n_out[i] = 0;
        return CSX_ERR_DEVICE_STATE;
    }
    return CSX_OK;
}

int csx_last_batch_info(csx_batch_info *out) {
    if (!out) return CSX_ERR_BAD_ARGS;
    Context *cx = nullptr;
    int rc = current_context(&cx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(cx->mu);
    *out = cx->binfo;
    return CSX_OK;
}

}  // extern "C"
