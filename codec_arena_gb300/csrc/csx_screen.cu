// csx_screen.cu — the GB300 screen funnel: src/screen.zig:run as a pipeline
// of sm_103a kernels behind the C ABI of include/csx_screen.h.
//
// Work decomposition. The reference runs T splitmix64 streams, stream t
// producing my_t candidates sequentially (src/screen.zig:273-297). A
// candidate consumes 33, 35, 62 or 64 draws, so where candidate i starts in
// its stream is only known by walking the stream. The pipeline:
//
//  1. walk    one thread per segment of L draws: follow the chain of
//             candidate starts from the segment's first draw (a guess), record
//             a checkpoint every D candidates, then follow this chain and the
//             next segment's guess chain in tandem until they meet. Two chains
//             that share a position coincide from there on; the first
//             segment's chain starts at draw 0 and is the true one, so the
//             truth is recovered segment by segment at the meeting points.
//  2. assemble one thread per stream: turn meeting points into the true
//             candidate range of every segment and its stream-local indices.
//  3. scan + emit  work items of <= D candidates with known start draw and
//             stream-local index, in (stream, index) order.
//  4. screen  persistent CTAs pull items; each thread synthesises and scores
//             candidates in registers; those that beat the CTA's threshold go
//             to a shared-memory buffer that is merged into the CTA's sorted
//             top-K list (bitonic sort). HBM sees only items and survivors.
//  5. merge   a tree of pairwise bitonic merges reduces the CTA lists.
//  6. regen   the K survivors are re-synthesised from (stream, draw) to
//             recover genes and lineage; the score is re-checked bit for bit.
//
// The walk costs two to three hashes per candidate against ~64 for
// synthesis. When streams are no longer than one item, steps 1-3 are skipped.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/csx_screen.h"
#include "csx_device.cuh"
#include "csx_tc.cuh"

namespace csx {

constexpr int kThreads = 256;      // screen CTA
constexpr int kRounds = 16;        // candidates per thread between CTA barriers
constexpr uint32_t kMaxKeep = 4096;
constexpr uint32_t kMaxElites = 1536;
constexpr uint64_t kLinkCap = 1ull << 26;
constexpr uint32_t kDefaultSegCands = 65536;

enum : uint32_t { kErrLink = 1u, kErrAssemble = 2u, kErrRegen = 4u, kErrItems = 8u };
enum : uint32_t { kSegOk = 0, kSegLast = 1, kSegFail = 2 };

struct Item {
    uint64_t draw0;   // first draw of the item's first candidate
    uint64_t idx0;    // stream-local index of that candidate
    uint32_t stream;
    uint32_t n;       // candidates in the item
};

// Top-K entry, ordered by (k1, k2) descending:
//   k1 = okey(score) << 32 | ~item,  k2 = ~dcand << 32 | ddraw
// so ties on the score go to the lower (stream, index). Zero is padding.
struct Entry {
    unsigned long long k1, k2;
};

// A candidate waiting for a second, more exact score (its item, its index in
// the item, its draw offset): the queues of the filter and precision forms.
struct Pend {
    uint32_t item, dcand, ddraw;
};
constexpr uint32_t kPendCap = 512;  // queue entries per CTA

struct SegRec {
    uint64_t merge_pos;  // first draw shared by this chain and the next segment's
    uint32_t n;          // chain candidates starting inside the segment
    uint32_t a;          // chain candidates from the segment end to merge_pos
    uint32_t b_next;     // next segment's chain candidates before merge_pos
    uint32_t status;
};

struct SegOut {
    uint64_t pos;   // draw of the first true candidate in this segment
    uint64_t I;     // its stream-local index
    uint64_t lo;    // its index along the segment's chain
    uint32_t cnt;   // true candidates taken from this segment
    uint32_t nitems;
};

struct Ctrl {
    unsigned int next_item;
    unsigned int gtau;  // best CTA threshold key seen so far (score okey)
    unsigned int err;
    unsigned int n_items;
    unsigned long long screened;
    unsigned long long n_out;
    unsigned long long exact_evals;  // reference-order evaluations (filter mode)
};

// Streams of one screen: T in all (src/screen.zig:267), of which this call
// walks and screens the contiguous range [t0, t0 + nT) (all of them unless a
// caller shards a generation by stream). Segment s is local to the range.
struct StreamGeom {
    uint64_t seed, T, per, my_last, L, n_seg, t0, nT;
    uint32_t C, C_last, d_log2, ckcap;
};

__device__ __forceinline__ bool better(const Entry &a, const Entry &b) {
    return a.k1 > b.k1 || (a.k1 == b.k1 && a.k2 > b.k2);
}

// Segment s of the range -> global stream t and segment c within it.
__device__ __forceinline__ void seg_of(const StreamGeom &g, uint64_t s, uint64_t &t, uint32_t &c) {
    t = s / g.C;
    if (t > g.nT - 1) t = g.nT - 1;
    c = static_cast<uint32_t>(s - t * g.C);
    t += g.t0;
}

__device__ __forceinline__ uint64_t stream_seed(uint64_t seed, uint64_t t) {
    return seed ^ (kGolden * (t + 1));  // src/screen.zig:284
}

// Split points m*D with lo < m*D < lo + cnt that have a checkpoint (m < ckcap).
__device__ __forceinline__ void split_range(uint64_t lo, uint64_t cnt, uint32_t dl, uint32_t ckcap,
                                            uint64_t &mmin, uint64_t &mmax) {
    mmin = (lo >> dl) + 1;
    mmax = (lo + cnt - 1) >> dl;
    if (mmax > static_cast<uint64_t>(ckcap) - 1) mmax = static_cast<uint64_t>(ckcap) - 1;
}

// ---- 0. elite table ---------------------------------------------------------

// (ne + 1) x 29 table, row ne = 0.5 (the immigrant row). -0.0 genes become
// +0.0, so clamp01 of a crossover gene never sees -0.0; NaN genes become +inf:
// the reference's clamp01(NaN + d) is 1 (@min returns the non-NaN operand),
// and so is clamp01(inf + d) for the finite d of the fast delta form, whose
// clamp the compiler may emit as a saturating add that flushes NaN to 0.
__global__ void prep_elites_kernel(const csx_genome *__restrict__ el, int ne, float *__restrict__ tab,
                                   unsigned long long *__restrict__ ids, unsigned int *__restrict__ tribes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ne * kNtot) {
        const int r = i / kNtot, k = i - r * kNtot;
        const float v = el[r].g[k];
        tab[i] = (v != v) ? INFINITY : __fadd_rn(v, 0.0f);
    } else if (i < (ne + 1) * kNtot) {
        tab[i] = 0.5f;
    }
    if (i < ne) {
        ids[i] = el[i].id;
        tribes[i] = el[i].tribe;
    }
}

// ---- 1. walk ------------------------------------------------------------------

// One thread per segment: the segment's guess chain from its first draw to
// its first start at or past the segment end, a checkpoint every D starts.
__global__ void walk_kernel(SynthConst sc, StreamGeom g, SegRec *__restrict__ recs,
                            uint64_t *__restrict__ ck, Ctrl *__restrict__ ctrl) {
    const uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= g.n_seg) return;
    uint64_t t;
    uint32_t c;
    seg_of(g, s, t, c);
    const bool last_stream = t == g.T - 1;
    const uint64_t my = last_stream ? g.my_last : g.per;
    const uint32_t ct = last_stream ? g.C_last : g.C;
    const uint64_t seed_t = stream_seed(g.seed, t);
    const uint64_t b = static_cast<uint64_t>(c) * g.L, e = b + g.L;
    uint64_t *ckp = ck + s * g.ckcap;
    const uint64_t dmask = (1ull << g.d_log2) - 1;
    uint64_t p = b, k = 0;
    const uint64_t limit = (ct == 1) ? my : ~0ull;  // a lone segment starts at the truth
    while (p < e && k < limit) {
        if ((k & dmask) == 0) {
            const uint64_t m = k >> g.d_log2;
            if (m < g.ckcap) ckp[m] = p;
        }
        p = walk_step2(sc, seed_t, p);
        ++k;
    }
    SegRec r;
    r.n = static_cast<uint32_t>(k);
    r.a = 0;
    r.b_next = 0;
    r.merge_pos = p;  // the chain's first start at or past the segment end
    r.status = (c + 1 == ct) ? kSegLast : kSegOk;
    recs[s] = r;
}

// Speculative run of one chain by a half-warp: lane j tests the start x + 62 j
// assuming every earlier step of the run is the common 62-draw one (no
// immigrant, no jump). f = first lane whose tests say otherwise (16 if none);
// the run's starts are x + 62 i for i <= min(f, 15) and the next start after
// it is x + 62 f + len (or x + 62*16).
struct Run {
    uint32_t n;     // starts in the run
    uint64_t next;  // the chain's next start after the run
};

__device__ __forceinline__ Run half_run(const SynthConst &C, uint64_t seed_t, uint64_t x, int j, int half) {
    const uint64_t pj = x + 62ull * static_cast<uint64_t>(j);
    const uint64_t s0 = seed_t + (pj + 1) * kGolden;               // state of draw pj
    const bool imm = (draw_vh(s0 + 2 * kGolden) >> 8) < C.imm_thr;  // draw pj + 2
    const bool jb = (draw_vh(s0 + 61 * kGolden) >> 8) < C.jump_thr; // draw pj + 61
    const uint32_t bn = (__ballot_sync(0xffffffffu, imm || jb) >> (16 * half)) & 0xffffu;
    const uint32_t bi = (__ballot_sync(0xffffffffu, imm) >> (16 * half)) & 0xffffu;
    Run r;
    if (bn == 0) {
        r.n = 16;
        r.next = x + 62ull * 16;
        return r;
    }
    const uint32_t f = static_cast<uint32_t>(__ffs(bn) - 1);
    const uint64_t pf = x + 62ull * f;
    uint32_t len = 64;            // a jump after a crossover candidate
    if ((bi >> f) & 1u) {         // an immigrant: its jump test is at draw + 32
        const bool ja = (draw_vh(seed_t + (pf + 33) * kGolden) >> 8) < C.jump_thr;
        len = ja ? 35 : 33;
    }
    r.n = f + 1;
    r.next = pf + len;
    return r;
}

// Checkpoint (start of every D-th candidate) among the starts [k, k + cnt),
// which lie at x + 62 (idx - k); D >= 64 > cnt, so at most one.
__device__ __forceinline__ void record_ckpt(uint64_t *ckp, uint32_t ckcap, uint32_t dl, uint64_t k,
                                            uint64_t cnt, uint64_t x) {
    const uint64_t mk = ((k + (1ull << dl) - 1) >> dl) << dl;
    if (mk < k + cnt && (mk >> dl) < ckcap) ckp[mk >> dl] = x + 62ull * (mk - k);
}

// One warp per link of segment s and s+1 (same stream): s's chain from its
// exit (lanes 0-15) and s+1's guess chain from its first draw (lanes 16-31)
// advance together in speculative runs. Below M = the nearer of the two next
// starts both chains' starts are known, and within a run they are 62 apart,
// so the first shared start below M is y if (y - x) is a multiple of 62
// inside x's run (or symmetrically). Otherwise both move to their first start
// at or past M and the search goes on.
__global__ void link_kernel(SynthConst sc, StreamGeom g, SegRec *__restrict__ recs,
                            uint64_t *__restrict__ ck, Ctrl *__restrict__ ctrl) {
    const int lane = threadIdx.x & 31, half = lane >> 4, j = lane & 15;
    const uint64_t s = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (s >= g.n_seg) return;  // whole warps leave together
    SegRec r = recs[s];
    if (r.status != kSegOk) return;
    uint64_t t;
    uint32_t c;
    seg_of(g, s, t, c);
    const uint64_t seed_t = stream_seed(g.seed, t);
    uint64_t *ckp = ck + s * g.ckcap;
    uint64_t x = r.merge_pos, k = r.n;                        // chain of segment s
    uint64_t y = static_cast<uint64_t>(c + 1) * g.L, kb = 0;  // guess chain of s + 1
    uint64_t steps = 0;
    bool fail = false;
    while (x != y) {
        const Run mine = half_run(sc, seed_t, half ? y : x, j, half);
        Run rx, ry;
        rx.n = __shfl_sync(0xffffffffu, mine.n, 0);
        rx.next = __shfl_sync(0xffffffffu, mine.next, 0);
        ry.n = __shfl_sync(0xffffffffu, mine.n, 16);
        ry.next = __shfl_sync(0xffffffffu, mine.next, 16);
        const uint64_t m = rx.next < ry.next ? rx.next : ry.next;
        // starts below m: x + 62 i for i < ix, y + 62 i for i < iy. Both chains
        // lie within a run (< 17 * 64 draws) of each other and of m, so the
        // differences fit 32 bits.
        const uint32_t ix = m > x ? min(rx.n, (static_cast<uint32_t>(m - x) + 61u) / 62u) : 0u;
        const uint32_t iy = m > y ? min(ry.n, (static_cast<uint32_t>(m - y) + 61u) / 62u) : 0u;
        bool met = false;
        uint32_t adv_x = ix, adv_y = iy;
        const uint32_t d = static_cast<uint32_t>(x < y ? y - x : x - y);
        const uint32_t dq = d / 62u;
        if (dq * 62u == d) {  // the leading start is on the lagging chain's run?
            if (x < y && dq < ix) {
                met = true;
                adv_x = dq;
                adv_y = 0;
            } else if (x > y && dq < iy) {
                met = true;
                adv_x = 0;
                adv_y = dq;
            }
        }
        if (lane == 0) record_ckpt(ckp, g.ckcap, g.d_log2, k, adv_x, x);
        const uint64_t nx = met ? x + 62ull * adv_x : (ix == rx.n ? rx.next : x + 62ull * ix);
        const uint64_t ny = met ? y + 62ull * adv_y : (iy == ry.n ? ry.next : y + 62ull * iy);
        k += adv_x;
        kb += adv_y;
        x = nx;
        y = ny;
        steps += adv_x + adv_y;
        if (steps > kLinkCap) {
            fail = true;
            break;
        }
    }
    if (lane == 0) {
        if (fail) {
            r.status = kSegFail;
            atomicOr(&ctrl->err, kErrLink);
        }
        r.merge_pos = x;
        r.a = static_cast<uint32_t>(k - r.n);
        r.b_next = static_cast<uint32_t>(kb);
        recs[s] = r;
    }
}

// ---- 2. assemble ------------------------------------------------------------------

__global__ void assemble_kernel(StreamGeom g, const SegRec *__restrict__ recs, SegOut *__restrict__ outs,
                                Ctrl *__restrict__ ctrl) {
    const uint64_t tl = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tl >= g.nT) return;
    const uint64_t t = g.t0 + tl;
    const bool last_stream = t == g.T - 1;
    const uint64_t my = last_stream ? g.my_last : g.per;
    const uint32_t ct = last_stream ? g.C_last : g.C;
    const uint64_t s0 = tl * g.C;
    uint64_t lo = 0, pos = 0, idx = 0;
    bool bad = false;
    for (uint32_t c = 0; c < ct; ++c) {
        const SegRec r = recs[s0 + c];
        SegOut o;
        o.pos = pos;
        o.I = idx;
        o.lo = lo;
        o.cnt = 0;
        o.nitems = 0;
        if (r.status == kSegFail) bad = true;
        const uint64_t hi = (r.status == kSegLast) ? r.n : static_cast<uint64_t>(r.n) + r.a;
        if (!bad && idx < my && hi > lo) {
            uint64_t cnt = hi - lo;
            if (cnt > my - idx) cnt = my - idx;
            uint64_t mmin, mmax;
            split_range(lo, cnt, g.d_log2, g.ckcap, mmin, mmax);
            o.cnt = static_cast<uint32_t>(cnt);
            o.nitems = 1 + (mmax >= mmin ? static_cast<uint32_t>(mmax - mmin + 1) : 0u);
            idx += cnt;
        }
        outs[s0 + c] = o;
        if (r.status == kSegOk) {
            if (hi >= lo) {  // the truth reaches the meeting point along this chain
                lo = r.b_next;
                pos = r.merge_pos;
            } else {         // the truth joined this chain after it met the next one
                lo = r.b_next + (lo - hi);
            }
        }
    }
    if (idx != my) atomicOr(&ctrl->err, kErrAssemble);
}

// One CTA per stream, 256 segments per tile. Segment c's truth range starts
// where link c-1 met (lo = b_next of c-1, pos = its merge_pos) unless segment
// c-1 was late: the truth reached c-1's chain only after that chain had met
// c's (lo > hi at c-1); then c's start is carried over (lo = b_next of c-1 +
// lo - hi of c-1, same pos). Late segments are rare and isolated, so the
// block computes the common case in parallel and thread 0 repairs the short
// runs after each late segment, carrying a pending state into the next tile.
constexpr int kAsmThreads = 256;

__global__ void __launch_bounds__(kAsmThreads) assemble_block_kernel(StreamGeom g,
                                                                      const SegRec *__restrict__ recs,
                                                                      SegOut *__restrict__ outs,
                                                                      Ctrl *__restrict__ ctrl) {
    __shared__ unsigned long long wsum[kAsmThreads / 32];
    __shared__ uint64_t s_lo[kAsmThreads], s_pos[kAsmThreads], s_hi[kAsmThreads];
    __shared__ uint32_t s_late[kAsmThreads / 32];
    __shared__ unsigned long long carry;
    __shared__ int pending, failed;
    __shared__ uint64_t pend_lo, pend_pos;
    const uint64_t tl = blockIdx.x, t = g.t0 + tl;
    const bool last_stream = t == g.T - 1;
    const uint64_t my = last_stream ? g.my_last : g.per;
    const uint32_t ct = last_stream ? g.C_last : g.C;
    const uint64_t s0 = tl * g.C;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) {
        carry = 0;
        pending = 0;
        failed = 0;
    }
    __syncthreads();
    for (uint32_t base = 0; base < ct; base += kAsmThreads) {
        const uint32_t c = base + tid;
        bool late = false, bad = false;
        if (c < ct) {
            const SegRec r = recs[s0 + c];
            uint64_t lo = 0, pos = 0;
            if (c > 0) {
                const SegRec q = recs[s0 + c - 1];
                lo = q.b_next;
                pos = q.merge_pos;
                bad |= q.status == kSegFail;
            }
            const uint64_t hi = (r.status == kSegLast) ? r.n : static_cast<uint64_t>(r.n) + r.a;
            bad |= r.status == kSegFail;
            late = lo > hi;
            s_lo[tid] = lo;
            s_pos[tid] = pos;
            s_hi[tid] = hi;
        }
        const uint32_t lb = __ballot_sync(0xffffffffu, late);
        if (lane == 0) s_late[w] = lb;
        if (__syncthreads_or(bad) && tid == 0) failed = 1;
        if (tid == 0) {  // repair the runs that follow late segments, in order
            const uint32_t n_here = min(static_cast<uint32_t>(kAsmThreads), ct - base);
            constexpr uint32_t kNone = 0xffffffffu;
            uint32_t x = kNone, from = 0;
            if (pending) {  // the previous tile ended inside a run
                s_lo[0] = pend_lo;
                s_pos[0] = pend_pos;
                pending = 0;
                x = 0;
            }
            for (;;) {
                if (x == kNone) {  // next flagged segment at or after `from`
                    for (uint32_t q = from >> 5; q < kAsmThreads / 32 && x == kNone; ++q) {
                        uint32_t bits = s_late[q];
                        if (q == (from >> 5)) bits &= ~((1u << (from & 31)) - 1u);
                        if (bits) x = q * 32 + __ffs(bits) - 1;
                    }
                    if (x == kNone || x >= n_here) break;
                }
                // x's state is its true one; carry while it is late
                while (s_lo[x] > s_hi[x]) {
                    const SegRec r = recs[s0 + base + x];
                    const uint64_t nlo = static_cast<uint64_t>(r.b_next) + (s_lo[x] - s_hi[x]);
                    if (x + 1 < n_here) {
                        s_lo[x + 1] = nlo;
                        s_pos[x + 1] = s_pos[x];
                        ++x;
                    } else {
                        if (base + x + 1 < ct) {
                            pending = 1;
                            pend_lo = nlo;
                            pend_pos = s_pos[x];
                        }
                        break;
                    }
                }
                from = x + 1;
                x = kNone;
                if (from >= n_here) break;
            }
        }
        __syncthreads();
        uint64_t lo = 0, pos = 0, len = 0;
        if (c < ct) {
            lo = s_lo[tid];
            pos = s_pos[tid];
            len = s_hi[tid] > lo ? s_hi[tid] - lo : 0;
        }
        // block exclusive scan of len
        unsigned long long v = len;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        if (lane == 31) wsum[w] = v;
        __syncthreads();
        if (w == 0) {
            unsigned long long x = lane < kAsmThreads / 32 ? wsum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long u = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += u;
            }
            if (lane < kAsmThreads / 32) wsum[lane] = x;
        }
        __syncthreads();
        const unsigned long long idx = carry + (w > 0 ? wsum[w - 1] : 0ull) + v - len;
        if (c < ct) {
            SegOut o;
            o.pos = pos;
            o.I = idx < my ? idx : my;
            o.lo = lo;
            o.cnt = 0;
            o.nitems = 0;
            if (!failed && idx < my && len > 0) {
                const uint64_t cnt = len < my - idx ? len : my - idx;
                uint64_t mmin, mmax;
                split_range(lo, cnt, g.d_log2, g.ckcap, mmin, mmax);
                o.cnt = static_cast<uint32_t>(cnt);
                o.nitems = 1 + (mmax >= mmin ? static_cast<uint32_t>(mmax - mmin + 1) : 0u);
            }
            outs[s0 + c] = o;
        }
        __syncthreads();
        if (tid == kAsmThreads - 1) carry += wsum[kAsmThreads / 32 - 1];
        __syncthreads();
    }
    if (tid == 0 && (failed || carry < my)) atomicOr(&ctrl->err, kErrAssemble);
}

// ---- 3. scan + emit ---------------------------------------------------------------

// Exclusive scan of SegOut::nitems by one CTA of 1024 threads (contiguous
// chunk per thread, then a block scan of the chunk sums).
__global__ void __launch_bounds__(1024) scan_kernel(const SegOut *__restrict__ outs, uint64_t n,
                                                    uint32_t *__restrict__ off, Ctrl *__restrict__ ctrl,
                                                    uint64_t items_cap) {
    __shared__ unsigned long long wsum[32];
    const uint32_t tid = threadIdx.x;
    const uint64_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint64_t b = tid * per, e = min(n, b + per);
    unsigned long long local = 0;
    for (uint64_t i = b; i < e; ++i) local += outs[i].nitems;
    // block exclusive scan of `local`
    unsigned long long v = local;
    const int lane = tid & 31, w = tid >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    if (w == 0) {
        unsigned long long x = lane < static_cast<int>(blockDim.x >> 5) ? wsum[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += u;
        }
        wsum[lane] = x;
    }
    __syncthreads();
    unsigned long long base = (w > 0 ? wsum[w - 1] : 0ull) + v - local;
    for (uint64_t i = b; i < e; ++i) {
        off[i] = static_cast<uint32_t>(base);
        base += outs[i].nitems;
    }
    if (tid == blockDim.x - 1) {
        if (base > items_cap || base >= 0xFFFFFFFFull) {
            atomicOr(&ctrl->err, kErrItems);
            base = 0;
        }
        ctrl->n_items = static_cast<unsigned int>(base);
    }
}

__global__ void emit_kernel(StreamGeom g, const SegOut *__restrict__ outs, const uint32_t *__restrict__ off,
                            const uint64_t *__restrict__ ck, Item *__restrict__ items,
                            const Ctrl *__restrict__ ctrl) {
    const uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= g.n_seg) return;
    const SegOut o = outs[s];
    if (o.cnt == 0 || (ctrl->err & kErrItems)) return;
    uint64_t t;
    uint32_t c;
    seg_of(g, s, t, c);
    const uint64_t *ckp = ck + s * g.ckcap;
    uint32_t j = off[s];
    uint64_t cur_lo = o.lo, cur_pos = o.pos, cur_i = o.I;
    const uint64_t end = o.lo + o.cnt;
    uint64_t mmin, mmax;
    split_range(o.lo, o.cnt, g.d_log2, g.ckcap, mmin, mmax);
    for (uint64_t m = mmin; m <= mmax; ++m) {
        const uint64_t nxt = m << g.d_log2;
        Item it;
        it.draw0 = cur_pos;
        it.idx0 = cur_i;
        it.stream = static_cast<uint32_t>(t);
        it.n = static_cast<uint32_t>(nxt - cur_lo);
        items[j++] = it;
        cur_i += nxt - cur_lo;
        cur_lo = nxt;
        cur_pos = ckp[m];
    }
    Item it;
    it.draw0 = cur_pos;
    it.idx0 = cur_i;
    it.stream = static_cast<uint32_t>(t);
    it.n = static_cast<uint32_t>(end - cur_lo);
    items[j] = it;
}

// Streams no longer than one item: one item per stream, starting at draw 0.
__global__ void stream_items_kernel(StreamGeom g, Item *__restrict__ items, Ctrl *__restrict__ ctrl) {
    const uint64_t tl = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tl == 0) ctrl->n_items = static_cast<unsigned int>(g.nT);
    if (tl >= g.nT) return;
    const uint64_t t = g.t0 + tl;
    Item it;
    it.draw0 = 0;
    it.idx0 = 0;
    it.stream = static_cast<uint32_t>(t);
    it.n = static_cast<uint32_t>(t == g.T - 1 ? g.my_last : g.per);
    items[tl] = it;
}

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
};

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
// finite): every candidate scored in the reference's f32 order.
template <bool kFastDelta>
__global__ void __launch_bounds__(kThreads, 3) screen_kernel(const __grid_constant__ ScreenArgs A) {
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
            const float s = synth_score<kFastDelta, false>(A.m, A.sc, el, seed_t, p, h, nullptr);
            if (s >= ts) {
                const unsigned long long k1 =
                    (static_cast<unsigned long long>(score_okey(s)) << 32) | static_cast<unsigned int>(~item);
                const unsigned long long k2 =
                    (static_cast<unsigned long long>(~dcand) << 32) | ddraw;
                if (k1 > t1 || (k1 == t1 && k2 > t2)) {
                    const unsigned int slot = atomicAdd(&s_buf_n, 1u);
                    if (slot < A.buf_cap) {
                        buf[slot] = Entry{k1, k2};
                    } else {
                        has_def = true;
                        def = Entry{k1, k2};
                    }
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
template <bool kFastDelta>
__global__ void __launch_bounds__(kThreads, 3) screen_q_kernel(const __grid_constant__ ScreenArgs A) {
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
            if (k1 > t1 || (k1 == t1 && k2 > t2)) buf[atomicAdd(&s_buf_n, 1u)] = Entry{k1, k2};
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
            if (s >= tlo) {
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
template <bool kFastDelta>
__device__ void regen_one(const DevModel &m, const SynthConst &sc, uint64_t seed, const float *el,
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
    const float s = synth_score<kFastDelta, true>(m, sc, el, seed_t, draw, h, genes);
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

__global__ void result_kernel(const Ctrl *__restrict__ ctrl, unsigned long long *__restrict__ result) {
    if (threadIdx.x == 0) {
        result[0] = ctrl->n_out;
        result[1] = ctrl->screened;
        result[2] = ctrl->err;
        result[3] = ctrl->n_items;
    }
}

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
        result;
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
};

Context g_ctx[64];

uint64_t env_u64(const char *name, uint64_t dflt) {
    const char *v = std::getenv(name);
    if (!v || !*v) return dflt;
    char *end = nullptr;
    const unsigned long long x = std::strtoull(v, &end, 10);
    return (end && *end == 0 && x > 0) ? x : dflt;
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
    (void)synth_score<kFastDelta, true, true>(*m, *sc, el, seed_t, p, h, g);
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
            if (k1 > t1 || (k1 == t1 && k2 > t2)) buf[atomicAdd(&s_buf_n, 1u)] = Entry{k1, k2};
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
            if (act) {
                const CandHead h = cand_head(A.sc, seed_t, p);
                synth_tc<kFastDelta, kFp16>(P.tm, A.sc, el, seed_t, p, h, R, x, pk);
                len = h.len;
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j) pk[j] = 0u;
#pragma unroll
                for (int i = 0; i < 16; ++i) x[i] = 0.0f;
            }
            float y[16];
            tc_ok = tc_round(tg, pk, tid & 127u, y) && tc_ok;
            if (act) {
                float s = R;
#pragma unroll
                for (int i = 0; i < 16; ++i) s = __fmaf_rn(x[i], y[i], s);
                if (s >= tlo) {
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

// grid_override, item_cands, seg_cands: 0 = automatic (the batched screen
// passes its own grid and the tuner's sizes).
int make_plan(const Context &cx, const csx_cfg &cfg, const csx_model &model, int ne, Plan *pl,
              int grid_override = 0, uint64_t item_cands = 0, uint64_t seg_cands = 0, uint64_t t_begin = 0,
              uint64_t t_end = 0) {
    StreamGeom &g = pl->g;
    g.seed = cfg.seed;
    g.T = std::max<uint64_t>(1, std::min<uint64_t>(cfg.threads, cfg.lambda));  // src/screen.zig:267
    g.per = cfg.lambda / g.T;
    g.my_last = cfg.lambda - (g.T - 1) * g.per;
    const uint64_t my_max = std::max(g.per, g.my_last);
    if (g.T >= 0xFFFFFFFFull) return CSX_ERR_LIMIT;
    if (t_end == 0) t_end = g.T;  // the whole generation
    if (t_begin >= t_end || t_end > g.T) return CSX_ERR_BAD_ARGS;
    g.t0 = t_begin;
    g.nT = t_end - t_begin;
    const bool has_last = t_end == g.T;
    const uint64_t lam_range = (g.nT - (has_last ? 1 : 0)) * g.per + (has_last ? g.my_last : 0);
    pl->fast_delta = std::isfinite(cfg.sigma) && std::fabs(cfg.sigma) <= 1.0e38f &&
                     (cfg.sigma == 0.0f || std::fabs(cfg.sigma) >= 1.0e-30f);
    pl->err = filter_bound(model);
    pl->filter = !(cfg.flags & CSX_FLAG_EXACT_ALL) && pl->err > 0.0f;

    pl->kpad = std::max<uint32_t>(32, pow2_at_least(cfg.keep));
    pl->sort_n = pow2_at_least(pl->kpad + 4ull * kThreads);
    pl->buf_cap = pl->sort_n - pl->kpad;
    const uint32_t tcf = cfg.flags & (CSX_FLAG_TC_BF16 | CSX_FLAG_TC_FP16);
    if (tcf == (CSX_FLAG_TC_BF16 | CSX_FLAG_TC_FP16)) return CSX_ERR_BAD_ARGS;
    pl->tc = tcf != 0;
    pl->fp16 = tcf == CSX_FLAG_TC_FP16;
    pl->smem = pl->tc ? static_cast<size_t>(pl->sort_n) * sizeof(Entry) +
                            static_cast<size_t>(ne + 1) * kNtot * sizeof(float) + kTcSmemExtra
                      : screen_smem(pl->sort_n, ne, pl->filter);
    if (pl->smem + 1024 > cx.max_smem) return CSX_ERR_LIMIT;
    if (grid_override > 0) {
        pl->grid = grid_override;
    } else if (pl->tc) {
        // The occupancy query reports one CTA per SM for this kernel, yet three
        // are resident and run faster (80 registers, ~50 KB of shared memory,
        // 32 TMEM columns each; measured). The screen is persistent with
        // dynamic work, so any grid is correct: launch three per SM.
        int rc = screen_occupancy(screen_tc_fn(pl->fast_delta, pl->fp16), cx.num_sms, pl->smem, &pl->grid);
        if (rc) return rc;
        pl->grid = kTcCtasPerSm * cx.num_sms;
    } else {
        int rc = screen_occupancy(screen_fn(pl->fast_delta, pl->filter), cx.num_sms, pl->smem, &pl->grid);
        if (rc) return rc;
    }

    // item size D: about 32 items per screen thread (measured: smaller items
    // shorten the tail of the persistent grid more than their reads cost)
    uint64_t d = item_cands ? item_cands : env_u64("CSX_ITEM_CANDS", 0);
    if (d == 0) {
        const uint64_t target = 32ull * static_cast<uint64_t>(pl->grid) * kThreads;
        d = std::max<uint64_t>(1, lam_range / target);
        d = std::min<uint64_t>(16384, std::max<uint64_t>(64, d));
    }
    uint32_t dl = 0;
    while ((2ull << dl) <= d) ++dl;  // D = 2^dl <= d
    g.d_log2 = dl;
    const uint64_t D = 1ull << dl;

    // candidate length is constant when neither branch probability is mixed
    const uint32_t it = unit_threshold(cfg.imm_p), jt = unit_threshold(cfg.jump_p);
    uint64_t gran = 2;
    if ((it == 0 || it == (1u << 24)) && (jt == 0 || jt == (1u << 24)))
        gran = (it ? 33 : 62) + (jt ? 2 : 0);
    const uint64_t seg = seg_cands ? seg_cands : env_u64("CSX_SEG_CANDS", kDefaultSegCands);
    uint64_t L = 64 * std::min(seg, my_max);
    L = ((L + gran - 1) / gran) * gran;
    g.L = L;
    g.C = static_cast<uint32_t>(std::max<uint64_t>(1, (64 * g.per + L - 1) / L));
    g.C_last = static_cast<uint32_t>(std::max<uint64_t>(1, (64 * g.my_last + L - 1) / L));
    g.n_seg = (g.nT - 1) * g.C + (has_last ? g.C_last : g.C);
    g.ckcap = static_cast<uint32_t>((2 * L / 33) / D + 3);
    pl->short_path = my_max <= D;
    pl->items_cap = pl->short_path ? g.nT : g.n_seg * (static_cast<uint64_t>(g.ckcap) + 1);
    if (pl->items_cap >= 0xFFFFFFFFull) return CSX_ERR_LIMIT;
    return CSX_OK;
}

int unit_blocks(uint64_t n, int threads) { return static_cast<int>((n + threads - 1) / threads); }

// Enqueue the whole pipeline on `st`. Device inputs: genomes (csx_genome x ne).
int enqueue_screen(Context &cx, const csx_cfg &cfg, const csx_model &model, const csx_genome *d_genomes,
                   int ne, csx_survivor *d_out, unsigned long long *d_result, cudaStream_t st,
                   uint64_t t_begin = 0, uint64_t t_end = 0) {
    Plan pl;
    int rc = make_plan(cx, cfg, model, ne, &pl, 0, 0, 0, t_begin, t_end);
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

    SynthConst sc;
    sc.ne = static_cast<uint32_t>(ne);
    sc.ne_magic = ~0ull / static_cast<uint64_t>(ne) + 1;
    sc.imm_thr = unit_threshold(cfg.imm_p);
    sc.jump_thr = unit_threshold(cfg.jump_p);
    sc.sigma = cfg.sigma;
    sc.nsig1 = -cfg.sigma;
    sc.sigma23 = cfg.sigma * 0x1p-23f;

    float *tab = static_cast<float *>(cx.tab.p);
    auto *ids = static_cast<unsigned long long *>(cx.ids.p);
    auto *tribes = static_cast<unsigned int *>(cx.tribes.p);
    prep_elites_kernel<<<unit_blocks(static_cast<uint64_t>(ne + 1) * kNtot, 256), 256, 0, st>>>(
        d_genomes, ne, tab, ids, tribes);
    CSX_CUDA(cudaGetLastError());
    ++launches;
    CSX_CUDA(mark(1));

    Item *items = static_cast<Item *>(cx.items.p);
    if (pl.short_path) {
        stream_items_kernel<<<unit_blocks(g.nT, 256), 256, 0, st>>>(g, items, ctrl);
        CSX_CUDA(cudaGetLastError());
        ++launches;
    } else {
        auto *recs = static_cast<SegRec *>(cx.recs.p);
        auto *ck = static_cast<uint64_t *>(cx.ck.p);
        auto *so = static_cast<SegOut *>(cx.segout.p);
        auto *off = static_cast<uint32_t *>(cx.off.p);
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
        launches += 5;
    }
    CSX_CUDA(mark(2));

    ScreenArgs A;
    A.m.w0 = model.w0;
    A.m.w16 = 16.0f * model.w0;
    for (int k = 0; k < kNtot; ++k) A.m.wlin[k] = model.w_lin[k];
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) A.m.wq[tri(i, j)] = model.w_quad[i * 16 + j];
    A.sc = sc;
    A.seed = cfg.seed;
    A.el = tab;
    A.items = items;
    A.ctrl = ctrl;
    A.lists = static_cast<Entry *>(cx.lists_a.p);
    A.keep = static_cast<uint32_t>(cfg.keep);
    A.kpad = pl.kpad;
    A.sort_n = pl.sort_n;
    A.buf_cap = pl.buf_cap;
    A.err = pl.err;
    if (pl.tc) {
        TcScreenArgs P;
        P.A = A;
        P.band = kTcBand;
        rc = make_tc_model(model, pl.fp16, &P.tm);
        if (rc) return rc;
        rc = tc_error_bound(model, pl.fp16, &P.err_abs);
        if (rc) return rc;
        screen_tc_fn(fast, pl.fp16)<<<pl.grid, kThreads, pl.smem, st>>>(P);
    } else {
        screen_fn(fast, pl.filter)<<<pl.grid, kThreads, pl.smem, st>>>(A);
    }
    CSX_CUDA(cudaGetLastError());
    ++launches;
    CSX_CUDA(mark(3));

    // merge tree
    const size_t msmem = 2ull * pl.kpad * sizeof(Entry);
    CSX_CUDA(cudaFuncSetAttribute(merge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(msmem)));
    Entry *cur = static_cast<Entry *>(cx.lists_a.p), *nxt = static_cast<Entry *>(cx.lists_b.p);
    uint32_t n = nl;
    while (n > 1) {
        const uint32_t m = (n + 1) / 2;
        merge_kernel<<<m, 256, msmem, st>>>(cur, n, nxt, pl.kpad);
        CSX_CUDA(cudaGetLastError());
        ++launches;
        std::swap(cur, nxt);
        n = m;
    }
    CSX_CUDA(mark(4));
    if (pl.tc && fast)
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

int csx_screen_device(const csx_cfg *cfg, const csx_model *model, const csx_genome *d_elites, int n_elites,
                      csx_survivor *d_out, uint64_t out_cap, uint64_t *d_result, void *cuda_stream) {
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
                          reinterpret_cast<unsigned long long *>(d_result), st);
}

}  // extern "C"

namespace csx {

// csx_screen / csx_screen_range: host buffers, a private stream, synchronous.
int screen_host(const csx_cfg *cfg, const csx_model *model, const csx_genome *elites, int n_elites,
                uint64_t t_begin, uint64_t t_end, csx_survivor *out, uint64_t out_cap, uint64_t *n_out,
                uint64_t *screened) {
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
        rc = enqueue_screen(*cx, *cfg, *model, dg, n_elites, ds, dr, st, t_begin, t_end);
        if (rc == CSX_OK) {
            e = cudaMemcpyAsync(res, dr, sizeof(res), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            const uint64_t cnt = std::min<uint64_t>(res[0], keep_n);
            if (e == cudaSuccess && res[2] == 0 && cnt > 0 && !(cfg->flags & CSX_FLAG_AS_SHIPPED)) {
                e = cudaMemcpyAsync(out, ds, cnt * sizeof(csx_survivor), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
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
int plan_noalloc(const NoAllocDevice &dv, const csx_cfg &cfg, const csx_model &model, int ne, Plan *pl) {
    StreamGeom &g = pl->g;
    g.seed = cfg.seed;
    g.T = std::max<uint64_t>(1, std::min<uint64_t>(cfg.threads, cfg.lambda));
    g.per = cfg.lambda / g.T;
    g.my_last = cfg.lambda - (g.T - 1) * g.per;
    g.t0 = 0;
    g.nT = g.T;
    const uint64_t my_max = std::max(g.per, g.my_last);
    if (g.T >= 0xFFFFFFFFull) return CSX_ERR_LIMIT;
    pl->fast_delta = std::isfinite(cfg.sigma) && std::fabs(cfg.sigma) <= 1.0e38f &&
                     (cfg.sigma == 0.0f || std::fabs(cfg.sigma) >= 1.0e-30f);
    pl->err = filter_bound(model);
    pl->filter = !(cfg.flags & CSX_FLAG_EXACT_ALL) && pl->err > 0.0f;
    pl->kpad = std::max<uint32_t>(32, pow2_at_least(cfg.keep));
    pl->sort_n = pow2_at_least(pl->kpad + 4ull * kThreads);
    pl->buf_cap = pl->sort_n - pl->kpad;
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
    const uint32_t it = unit_threshold(cfg.imm_p), jt = unit_threshold(cfg.jump_p);
    uint64_t gran = 2;
    if ((it == 0 || it == (1u << 24)) && (jt == 0 || jt == (1u << 24)))
        gran = (it ? 33 : 62) + (jt ? 2 : 0);
    uint64_t L = 64 * std::min<uint64_t>(kDefaultSegCands, my_max);
    L = ((L + gran - 1) / gran) * gran;
    g.L = L;
    g.C = static_cast<uint32_t>(std::max<uint64_t>(1, (64 * g.per + L - 1) / L));
    g.C_last = static_cast<uint32_t>(std::max<uint64_t>(1, (64 * g.my_last + L - 1) / L));
    g.n_seg = (g.T - 1) * g.C + g.C_last;
    g.ckcap = static_cast<uint32_t>((L / 33) / D + 3);
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
    SynthConst sc;
    sc.ne = static_cast<uint32_t>(ne);
    sc.ne_magic = ~0ull / static_cast<uint64_t>(ne) + 1;
    sc.imm_thr = unit_threshold(cfg.imm_p);
    sc.jump_thr = unit_threshold(cfg.jump_p);
    sc.sigma = cfg.sigma;
    sc.nsig1 = -cfg.sigma;
    sc.sigma23 = cfg.sigma * 0x1p-23f;
    prep_elites_kernel<<<unit_blocks(static_cast<uint64_t>(ne + 1) * kNtot, 256), 256, 0, st>>>(
        d_genomes, ne, tab, ids, tribes);
    CSX_CUDA(cudaGetLastError());
    if (pl.short_path) {
        stream_items_kernel<<<unit_blocks(g.nT, 256), 256, 0, st>>>(g, items, ctrl);
        CSX_CUDA(cudaGetLastError());
    } else {
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
    }
    ScreenArgs A;
    A.m.w0 = model.w0;
    A.m.w16 = 16.0f * model.w0;
    for (int k = 0; k < kNtot; ++k) A.m.wlin[k] = model.w_lin[k];
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) A.m.wq[tri(i, j)] = model.w_quad[i * 16 + j];
    A.sc = sc;
    A.seed = cfg.seed;
    A.el = tab;
    A.items = items;
    A.ctrl = ctrl;
    A.lists = lists_a;
    A.keep = static_cast<uint32_t>(cfg.keep);
    A.kpad = pl.kpad;
    A.sort_n = pl.sort_n;
    A.buf_cap = pl.buf_cap;
    A.err = pl.err;
    screen_fn(fast, pl.filter)<<<pl.grid, kThreads, pl.smem, st>>>(A);
    CSX_CUDA(cudaGetLastError());
    const size_t msmem = 2ull * pl.kpad * sizeof(Entry);
    CSX_CUDA(cudaFuncSetAttribute(merge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(msmem)));
    Entry *cur = lists_a, *nxt = lists_b;
    uint32_t n = nl;
    while (n > 1) {
        const uint32_t m = (n + 1) / 2;
        merge_kernel<<<m, 256, msmem, st>>>(cur, n, nxt, pl.kpad);
        CSX_CUDA(cudaGetLastError());
        std::swap(cur, nxt);
        n = m;
    }
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

// ---- batched islands -------------------------------------------------------------
//
// Several independent screens in one pipeline. Each island's items are built
// by the single-screen stages on a forked stream of its own (the stages of
// small islands are short of parallel work, so islands overlap). One
// persistent launch then screens every island's items: a global counter hands
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
            if (k1 > t1 || (k1 == t1 && k2 > t2)) E[s_kpad + atomicAdd(&s_buf_n, 1u)] = Entry{k1, k2};
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
                if (s >= tlo) {
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
            if (!kFilter && s >= ts) {
                const unsigned long long k1 =
                    (static_cast<unsigned long long>(score_okey(s)) << 32) | static_cast<unsigned int>(~item);
                const unsigned long long k2 = (static_cast<unsigned long long>(~dcand) << 32) | ddraw;
                if (k1 > t1 || (k1 == t1 && k2 > t2)) {
                    const unsigned int slot = atomicAdd(&s_buf_n, 1u);
                    if (slot < bcap) {
                        buf[slot] = Entry{k1, k2};
                    } else {
                        has_def = true;
                        def = Entry{k1, k2};
                    }
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

RowModel make_row_model(const DevModel &m) {
    RowModel r{};
    for (int k = 0; k < 16; ++k) {
        for (int l = 0; l <= k; ++l) r.v[row_off(k) + l] = m.wq[tri(k, l)];
        r.v[row_off(k) + k + 1] = m.wlin[k];
    }
    for (int k = 16; k < kNtot; ++k) r.v[kRowLin16 + k - 16] = m.wlin[k];
    r.v[kRowW16] = m.w16;
    r.v[kRowW16 + 1] = m.w0;
    return r;
}

DevModel make_dev_model(const csx_model &model) {
    DevModel m;
    m.w0 = model.w0;
    m.w16 = 16.0f * model.w0;
    for (int k = 0; k < kNtot; ++k) m.wlin[k] = model.w_lin[k];
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) m.wq[tri(i, j)] = model.w_quad[i * 16 + j];
    return m;
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
        const uint32_t kpad = std::max<uint32_t>(32, pow2_at_least(c.keep));
        L->kpad_max = std::max(L->kpad_max, kpad);
        L->keep_max = std::max<uint32_t>(L->keep_max, static_cast<uint32_t>(c.keep));
        L->sort_n = std::max(L->sort_n, pow2_at_least(kpad + 4ull * kThreads));
        ne_max = std::max(ne_max, n_elites[i]);
    }
    L->ne_max = static_cast<uint32_t>(ne_max);
    L->smem = screen_smem(L->sort_n, ne_max, L->filter);
    if (L->smem + 2048 > cx.max_smem) return CSX_ERR_LIMIT;
    BatchFn fn = batch_fn(L->fast, L->filter);
    CSX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(L->smem)));
    int per_sm = 0;
    CSX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, L->smem));
    per_sm = std::max(1, per_sm);
    if (tune && tune->ctas_per_sm > 0) per_sm = std::min<int>(per_sm, static_cast<int>(tune->ctas_per_sm));
    L->grid = per_sm * cx.num_sms;
    const size_t msmem = 2ull * L->kpad_max * sizeof(Entry);
    CSX_CUDA(cudaFuncSetAttribute(merge_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(msmem)));

    uint64_t items_sum = 0;
    for (int i = 0; i < n; ++i) {
        if (cfgs[i].lambda == 0) continue;
        int rc = make_plan(cx, cfgs[i], models[i], n_elites[i], &L->pl[i], L->grid, tune ? tune->item_cands : 0,
                           tune ? tune->seg_cands : 0);
        if (rc) return rc;
        items_sum += L->pl[i].items_cap;
    }
    if (items_sum >= 0xFFFFFFFFull) return CSX_ERR_LIMIT;

    // carve: a sizing pass, then the real one
    const uint32_t nl = static_cast<uint32_t>(L->grid);
    auto carve = [&](unsigned char *base) -> size_t {
        Carve cv{base};
        L->d_isl = cv.take<IslandDev>(n);
        L->d_base = cv.take<unsigned int>(n + 1);
        L->d_next = cv.take<unsigned int>(1);
        L->ctrl_all = cv.take<Ctrl>(n);
        const size_t lists0 = (cv.off + 255) & ~static_cast<size_t>(255);
        for (int i = 0; i < n; ++i) {
            const uint32_t kpad = std::max<uint32_t>(32, pow2_at_least(cfgs[i].keep));
            L->b[i].la = cv.take<Entry>(static_cast<size_t>(nl) * kpad);
        }
        L->lists_all = reinterpret_cast<Entry *>(base + lists0);
        L->lists_bytes = cv.off - lists0;
        for (int i = 0; i < n; ++i) {
            IslandBufs &b = L->b[i];
            const Plan &pl = L->pl[i];
            const uint32_t kpad = std::max<uint32_t>(32, pow2_at_least(cfgs[i].keep));
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
        d.kpad = std::max<uint32_t>(32, pow2_at_least(cfgs[i].keep));
        d.ne = static_cast<uint32_t>(n_elites[i]);
        d.err = filter_bound(models[i]);
        out_off += cfgs[i].keep;
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
            if (pl.short_path) {
                stream_items_kernel<<<unit_blocks(g.nT, 256), 256, 0, a>>>(g, b.items, b.ctrl);
                CSX_CUDA(cudaGetLastError());
                ++nk;
            } else {
                walk_kernel<<<unit_blocks(g.n_seg, 128), 128, 0, a>>>(sc, g, b.recs, b.ck, b.ctrl);
                CSX_CUDA(cudaGetLastError());
                link_kernel<<<unit_blocks(g.n_seg * 32, 128), 128, 0, a>>>(sc, g, b.recs, b.ck, b.ctrl);
                CSX_CUDA(cudaGetLastError());
                if (g.C >= 64)
                    assemble_block_kernel<<<static_cast<unsigned>(g.nT), kAsmThreads, 0, a>>>(g, b.recs, b.so, b.ctrl);
                else
                    assemble_kernel<<<unit_blocks(g.nT, 128), 128, 0, a>>>(g, b.recs, b.so, b.ctrl);
                CSX_CUDA(cudaGetLastError());
                scan_kernel<<<1, 1024, 0, a>>>(b.so, g.n_seg, b.off, b.ctrl, pl.items_cap);
                CSX_CUDA(cudaGetLastError());
                emit_kernel<<<unit_blocks(g.n_seg, 128), 128, 0, a>>>(g, b.so, b.off, b.ck, b.items, b.ctrl);
                CSX_CUDA(cudaGetLastError());
                nk += 5;
            }
        }
        CSX_CUDA(cudaEventRecord(cx.ev_join[i], a));
        CSX_CUDA(cudaStreamWaitEvent(st, cx.ev_join[i], 0));
    }
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
        ok = tc_round(g, pk, tid, y) && ok;
        float s = R;
#pragma unroll
        for (int i = 0; i < 16; ++i) s = __fmaf_rn(x[i], y[i], s);
        if (r < n) out[r] = s;
    }
    if (!ok) atomicOr(err, kErrTc);
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

}  // namespace csx

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
