// csx_ties.cuh — exact tie order: the device half of the replay of a
// stream's heap (src/screen.zig:151-193,306-319).
// Part of csx_screen.cu's translation unit (included there, in order); not a
// standalone header.
//
// The reference keeps each stream's top-K in a binary min-heap that rejects a
// candidate scoring <= its root, then stable-sorts the concatenated heap
// arrays by score. Candidates with exactly equal f32 scores from one stream
// therefore rank by their final heap-array positions, and at the K-th score
// the heap's history decides which of them survive. The screen ranks ties
// by (stream, index) instead; for the streams where that can differ the host
// replays the stream's heap (csx_screen.cu, fix_ties) from the candidates
// these kernels collect.
#pragma once

namespace csx {

// A candidate of the replayed stream: its stream-local index, first draw and
// reference-order score.
struct TieHit {
    uint64_t index, draw;
    float score;
    uint32_t pad_;
};

// Every candidate of stream `stream` with stream-local index in [a, b) whose
// score exceeds thr (all of them when `all`), appended to out (at most cap;
// *count counts every append, so a count above cap reports an overflow).
// One thread per work item of the generation; items of other streams or
// ranges return at once.
template <bool kFastDelta, class Args>
__global__ void tie_collect_kernel(const __grid_constant__ Args A, uint64_t n_items, uint32_t stream, uint64_t a,
                                   uint64_t b, float thr, int all, TieHit *__restrict__ out,
                                   unsigned int *__restrict__ count, unsigned int cap) {
    const uint64_t seed_t = stream_seed(A.seed, stream);
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n_items;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const Item it = A.items[i];
        if (it.stream != stream || it.idx0 >= b || it.idx0 + it.n <= a) continue;
        uint64_t p = it.draw0;
        for (uint32_t c = 0; c < it.n; ++c) {
            const uint64_t idx = it.idx0 + c;
            if (idx >= b) break;
            const CandHead h = cand_head(A.sc, seed_t, p);
            if (idx >= a) {
                const float s = cand_score<kFastDelta>(A, A.el, seed_t, p, h);
                if (all || s > thr) {
                    const unsigned int slot = atomicAdd(count, 1u);
                    if (slot < cap) out[slot] = TieHit{idx, p, s, 0u};
                }
            }
            p += h.len;
        }
    }
}

// Survivor records of the candidates at (stream, draw, index): genes and
// lineage regenerated, the score in the reference's order (the full
// surface's with FullScreenArgs).
template <bool kFastDelta, class Model>
__device__ void tie_regen_one(const Model &m, const SynthConst &sc, uint64_t seed, const float *el,
                              const unsigned long long *ids, const unsigned int *tribes, const TieHit &t,
                              uint64_t stream, csx_survivor *o) {
    const uint64_t seed_t = stream_seed(seed, stream);
    const CandHead h = cand_head(sc, seed_t, t.draw);
    float genes[kNtot];
    const float s = cand_genes<kFastDelta>(m, sc, el, seed_t, t.draw, h, genes);
    csx_survivor v;
    v.score = s;
    v.tribe = tribes[h.ea];
    v.pa = ids[h.ea];
    v.pb = ids[h.eb];
    v.stream = stream;
    v.index = t.index;
    v.draw = t.draw;
#pragma unroll
    for (int k = 0; k < kNtot; ++k) v.g[k] = genes[k];
    v.reserved = 0;
    *o = v;
}

template <bool kFastDelta>
__global__ void tie_regen_kernel(const __grid_constant__ ScreenArgs A, const TieHit *__restrict__ hits,
                                 const uint64_t *__restrict__ streams, uint32_t n,
                                 const unsigned long long *__restrict__ ids, const unsigned int *__restrict__ tribes,
                                 csx_survivor *__restrict__ out) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) tie_regen_one<kFastDelta>(A.m, A.sc, A.seed, A.el, ids, tribes, hits[q], streams[q], out + q);
}

template <bool kFastDelta>
__global__ void tie_regen_full_kernel(const __grid_constant__ FullScreenArgs A, const TieHit *__restrict__ hits,
                                      const uint64_t *__restrict__ streams, uint32_t n,
                                      const unsigned long long *__restrict__ ids,
                                      const unsigned int *__restrict__ tribes, csx_survivor *__restrict__ out) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) tie_regen_one<kFastDelta>(A.fm, A.sc, A.seed, A.el, ids, tribes, hits[q], streams[q], out + q);
}

}  // namespace csx
