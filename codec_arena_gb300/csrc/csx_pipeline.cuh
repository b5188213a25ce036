// csx_pipeline.cuh — types of the screen pipeline and its item-building
// kernels: the elite table, the walk of each stream's segments, the links
// between segments, the assembly of true candidate ranges, and the scan and
// emission of work items.
// Part of csx_screen.cu's translation unit (included there, in order); not a
// standalone header.
#pragma once

namespace csx {


constexpr int kThreads = 256;      // screen CTA
constexpr int kRounds = 16;        // candidates per thread between CTA barriers
constexpr uint32_t kMaxKeep = 4096;
constexpr uint32_t kMaxElites = 1536;
constexpr uint64_t kLinkCap = 1ull << 26;
// Candidates per walk segment: 49152 measured best for walk + link at 2.65e9
// (9.3 ms; 11.5 at 65536, 10.5 at 32768). The no-allocation entry keeps
// 65536 so that its static scratch holds the same configurations.
constexpr uint32_t kDefaultSegCands = 49152;
constexpr uint32_t kNoAllocSegCands = 65536;

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
    unsigned int item_begin;         // first item of this call's share (item sharding), else 0
    unsigned int pad_;
};

// Streams of one screen: T in all (src/screen.zig:267), of which this call
// walks and screens the contiguous range [t0, t0 + nT) (all of them unless a
// caller shards a generation by stream). Segment s is local to the range.
struct StreamGeom {
    uint64_t seed, T, per, my_last, L, n_seg, t0, nT;
    uint64_t link_cap;  // link steps before a boundary is declared failed (kLinkCap; CSX_LINK_CAP)
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
// The chain carries the splitmix64 state of its start beside the position
// and runs D steps between checkpoints with a 32-bit count (measured 5%
// faster than one loop testing for a checkpoint at every step).
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
    const uint32_t D = 1u << g.d_log2;
    // the position as the draws left to the segment end, a 32-bit count
    // (segments are at most 2^30 draws: segment_geometry)
    int32_t rem = static_cast<int32_t>(g.L);
    uint64_t k = 0;
    uint64_t st = seed_t + (b + 1) * kGolden;
    const uint64_t limit = (ct == 1) ? my : ~0ull;  // a lone segment starts at the truth
    while (rem > 0 && k < limit) {
        const uint64_t m = k >> g.d_log2;  // k is a multiple of D here
        if (m < g.ckcap) ckp[m] = e - static_cast<uint64_t>(rem);
        const uint32_t n = static_cast<uint32_t>(min(static_cast<uint64_t>(D), limit - k));
        uint32_t j = 0;
        do {
            const uint32_t len = cand_len(sc, st);
            rem -= static_cast<int32_t>(len);
            st += static_cast<uint64_t>(len) * kGolden;
            ++j;
        } while (j < n && rem > 0);
        k += j;
    }
    SegRec r;
    r.n = static_cast<uint32_t>(k);
    r.a = 0;
    r.b_next = 0;
    r.merge_pos = e + static_cast<uint64_t>(-static_cast<int64_t>(rem));  // the first start at or past the end
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

// The same speculative run by the whole warp: lane j tests x + 62 j, the run
// has up to 32 starts.
__device__ __forceinline__ Run warp_run(const SynthConst &C, uint64_t seed_t, uint64_t x, int lane) {
    const uint64_t pj = x + 62ull * static_cast<uint64_t>(lane);
    const uint64_t s0 = seed_t + (pj + 1) * kGolden;
    const bool imm = (draw_vh(s0 + 2 * kGolden) >> 8) < C.imm_thr;
    const bool jb = (draw_vh(s0 + 61 * kGolden) >> 8) < C.jump_thr;
    const uint32_t bn = __ballot_sync(0xffffffffu, imm || jb);
    const uint32_t bi = __ballot_sync(0xffffffffu, imm);
    Run r;
    if (bn == 0) {
        r.n = 32;
        r.next = x + 62ull * 32;
        return r;
    }
    const uint32_t f = static_cast<uint32_t>(__ffs(bn) - 1);
    const uint64_t pf = x + 62ull * f;
    uint32_t len = 64;
    if ((bi >> f) & 1u) {
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

// One warp per link of segment s and s+1 (same stream). Segment s's chain is
// followed from its exit in whole-warp speculative runs until it lands on one
// of the checkpoints the walk wrote for s+1's guess chain (every D-th start
// before s+1's exit): a chain that reaches a start of another follows it from
// there on, so the first checkpoint after the two chains meet is the first
// one s's chain lands on, and only s's chain is walked. (Walking both chains
// to their first shared start costs about four times the instructions.) If
// s's chain passes the last of those checkpoints first, the meeting lies past
// s+1's exit: the two chains then advance together, 16 lanes each, from s's
// position and that checkpoint. Below M = the nearer of the two next starts
// both chains' starts are known, and within a run they are 62 apart, so the
// first shared start below M is y if (y - x) is a multiple of 62 inside x's
// run (or symmetrically). Otherwise both move to their first start at or past
// M and the search goes on.
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
    uint64_t x = r.merge_pos, k = r.n;  // chain of segment s
    // s+1's walk checkpoints: starts m * D < n of s+1 (n is the walk's count;
    // the link of s+1 rewrites that record with the same n)
    const uint32_t n_next = *reinterpret_cast<volatile const uint32_t *>(&recs[s + 1].n);
    const uint64_t *cky = ck + (s + 1) * g.ckcap;
    const uint32_t D = 1u << g.d_log2;
    const uint32_t mcap = min(g.ckcap, (n_next + D - 1) >> g.d_log2);  // >= 1: a chain has a start
    uint32_t cm = 0;
    uint64_t cy = cky[0];
    while (cm + 1 < mcap && cy < x) cy = cky[++cm];
    uint64_t y = cy, kb = static_cast<uint64_t>(cm) << g.d_log2;  // guess chain of s + 1
    uint64_t steps = 0;
    bool fail = false;
    if (cy >= x) {
        for (;;) {
            const Run run = warp_run(sc, seed_t, x, lane);
            const uint64_t d = cy - x;  // < one checkpoint gap + a run: fits 32 bits
            const uint32_t dq = static_cast<uint32_t>(d) / 62u;
            if (static_cast<uint32_t>(d) == dq * 62u && dq < run.n) {  // lands on it
                if (lane == 0) record_ckpt(ckp, g.ckcap, g.d_log2, k, dq, x);
                k += dq;
                x = cy;
                break;
            }
            if (lane == 0) record_ckpt(ckp, g.ckcap, g.d_log2, k, run.n, x);
            k += run.n;
            x = run.next;
            steps += run.n;
            while (cy < x && cm + 1 < mcap) cy = cky[++cm];
            if (cy < x) {  // past the last checkpoint: meet beyond it (below)
                y = cy;
                kb = static_cast<uint64_t>(cm) << g.d_log2;
                break;
            }
            if (steps > g.link_cap) {
                fail = true;
                break;
            }
        }
        if (x == cy) {
            y = cy;
            kb = static_cast<uint64_t>(cm) << g.d_log2;
        }
    }
    while (x != y && !fail) {
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
        if (steps > g.link_cap) {
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
        // after a failed link or assembly no item is emitted or screened: the
        // stages that follow see n_items = 0 and the error bits void the call
        if (ctrl->err) base = 0;
        ctrl->n_items = static_cast<unsigned int>(base);
    }
}

__global__ void emit_kernel(StreamGeom g, const SegOut *__restrict__ outs, const uint32_t *__restrict__ off,
                            const uint64_t *__restrict__ ck, Item *__restrict__ items,
                            const Ctrl *__restrict__ ctrl) {
    const uint64_t s = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= g.n_seg) return;
    const SegOut o = outs[s];
    if (o.cnt == 0 || ctrl->err) return;
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
// Item sharding: this call screens items [n * shard / n_shards, n * (shard +
// 1) / n_shards) of the n the item stages emitted (the screen kernels pull
// items from next_item up to n_items).
__global__ void shard_items_kernel(Ctrl *ctrl, uint32_t shard, uint32_t n_shards) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const uint64_t n = ctrl->n_items;
        ctrl->item_begin = static_cast<unsigned int>(n * shard / n_shards);
        ctrl->next_item = ctrl->item_begin;
        ctrl->n_items = static_cast<unsigned int>(n * (shard + 1) / n_shards);
    }
}

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

}  // namespace csx
