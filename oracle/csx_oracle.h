/*
 * csx_oracle.h — CPU restatement of codec-arena's screen funnel.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity checker and the timed
 * CPU baseline. Only tests/, __graft_entry__.smoke() and bench.py (its CPU
 * baseline / reference arm) may load it. The product path (libcsx_screen.so)
 * never links or calls it.
 *
 * What it restates (reference paths are relative to the codec-arena tree):
 *   src/screen.zig:36-95    Model.fromCompact   -> orc_model_from_compact
 *   src/screen.zig:97-112   Model.score         -> orc_score (same f32 op order)
 *   src/screen.zig:115-127  loadModel           -> orc_model_parse
 *   src/screen.zig:151-193  Heap.offer          -> per-stream min-heap, `<=` reject
 *   src/screen.zig:195-213  Rng (splitmix64)    -> orc_splitmix_next / unit
 *   src/screen.zig:225-255  worker              -> orc_candidate (draw order)
 *   src/screen.zig:257-343  run                 -> orc_screen (streams, merge)
 *   src/genome.zig:116-188  parseLine           -> orc_parse_line
 *   src/genome.zig:292-294  clamp01
 *
 * Parity status: PARTIALLY PINNED. The reference is Zig and no Zig toolchain
 * is available, so it cannot be run to produce outputs. Pinned: the
 * compact->flat layout known answers (src/screen.zig:345-377), the score
 * monotonicity / neutrality test (src/screen.zig:379-405), the parse known
 * answers (src/genome.zig:296-372, with the v6 quirk below) and the published
 * splitmix64 output sequence. Unpinned (restated from reading the code): the
 * per-candidate draw order, heap tie behaviour and the merge order.
 *
 * Intended vs as-shipped semantics: run() copies each Heap into its worker by
 * value (src/screen.zig:221,285) so the merge reads heaps whose n is 0 and the
 * shipped binary writes an empty promoted file. The oracle implements the
 * intended merge (the workers' heaps); ORC_FLAG_AS_SHIPPED reproduces the
 * empty output.
 */
#ifndef CSX_ORACLE_H
#define CSX_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NG 23
#define ORC_NR 6
#define ORC_NTOT 29

/* flags (same bit values as the product's CSX_FLAG_* where they overlap) */
#define ORC_FLAG_AS_SHIPPED 0x1u   /* empty survivor list, as the shipped binary */
#define ORC_FLAG_PARSE_V6_FIX 0x4u /* 34-token lines keep genes 16..21 */

typedef struct orc_model {
    float w0;
    float w_lin[ORC_NTOT];
    float w_quad[256];
} orc_model;

typedef struct orc_genome {
    uint64_t id;
    uint64_t pa;
    uint64_t pb;
    uint32_t gen;
    uint32_t tribe;
    float g[ORC_NTOT]; /* 23 effectors then 6 regulators */
    uint32_t pad_;
} orc_genome;

typedef struct orc_cfg {
    uint64_t lambda;
    uint64_t keep;
    uint64_t seed;
    uint64_t threads;
    float sigma;
    float jump_p;
    float imm_p;
    uint32_t flags;
} orc_cfg;

typedef struct orc_survivor {
    float score;
    uint32_t tribe;
    uint64_t pa;
    uint64_t pb;
    uint64_t stream;
    uint64_t index; /* candidate index within its stream */
    uint64_t draw;  /* RNG draw position of the candidate's first draw */
    float g[ORC_NTOT];
    uint32_t pad_;
} orc_survivor;

enum {
    ORC_OK = 0,
    ORC_ERR_BAD_MODEL = -1,
    ORC_ERR_NEED_TWO_ELITES = -2,
    ORC_ERR_BAD_ARGS = -3,
    ORC_ERR_PARSE = -4,
    ORC_ERR_OOM = -9,
};

uint64_t orc_splitmix_next(uint64_t *state);
uint64_t orc_stream_seed(uint64_t seed, uint64_t t);
int orc_model_from_compact(const float *w, int n, orc_model *m);
int orc_model_parse(const char *txt, size_t len, float *w, int cap, int *n_out);
float orc_score(const orc_model *m, const float *g);
double orc_score_f64(const orc_model *m, const float *g);
int orc_parse_line(const char *line, size_t len, uint32_t flags, orc_genome *out);
int orc_elites_parse(const char *txt, size_t len, uint32_t flags, orc_genome *out,
                     int cap, int *n_out);

/* Synthesise the candidate whose first draw is `draw` in stream t. Fills
 * genes, lineage and the f32 score; *next_draw = first draw of the next one. */
void orc_candidate(const orc_cfg *cfg, const orc_model *m, const orc_genome *el,
                   int ne, uint64_t t, uint64_t draw, orc_survivor *out,
                   uint64_t *next_draw);

/* Dump n candidates of stream t starting at candidate 0 (small tests). */
int orc_stream_dump(const orc_cfg *cfg, const orc_model *m, const orc_genome *el,
                    int ne, uint64_t t, uint64_t n, orc_survivor *out);

/* run(): T splitmix64 streams, a `keep`-slot heap per stream, the intended
 * merge, stable sort by score desc. cpu_threads OS threads share the streams
 * (0 = one per stream up to 64). Survivors are written to out[0..*n_out). */
int orc_screen(const orc_cfg *cfg, const orc_model *m, const orc_genome *el, int ne,
               int cpu_threads, orc_survivor *out, uint64_t out_cap, uint64_t *n_out,
               uint64_t *screened);

/* ---- full quadratic surface ----------------------------------------------
 * No reference code: docs/RESEARCH_V05C.md:99-102 queues a surrogate whose
 * quadratic block covers all 29 genes ("extend the quad block in v0.6").
 * Compact layout (ORC_FULL_NF = 465 floats): [0] constant, [1..29] linear
 * terms, then g_i*g_j for j <= i < 29, i outer, j inner -- the v6 layout's
 * quadratic block extended from 16 to 29 genes. The f32 score is defined by
 * this FMA order (one rounding per fmaf):
 *   r = w0; for k in 0..28: t = w_lin[k]; for l in 0..k: t = fmaf(Q[k][l], g[l], t);
 *                           r = fmaf(g[k], t, r)
 * i.e. w0 + sum_k g_k (w_k + sum_{l<=k} Q_kl g_l), the intercept counted once. */
#define ORC_FULL_NF 465
#define ORC_FULL_NQ 435

typedef struct orc_model_full {
    float w0;
    float w_lin[ORC_NTOT];
    float w_quad[ORC_FULL_NQ]; /* (i, j <= i) at i*(i+1)/2 + j */
} orc_model_full;

int orc_model_full_from_compact(const float *w, int n, orc_model_full *m);
float orc_score_full(const orc_model_full *m, const float *g);
double orc_score_full_f64(const orc_model_full *m, const float *g);
/* orc_candidate / orc_screen with the full surface scoring the candidates. */
void orc_candidate_full(const orc_cfg *cfg, const orc_model_full *m, const orc_genome *el, int ne,
                        uint64_t t, uint64_t draw, orc_survivor *out, uint64_t *next_draw);
int orc_screen_full(const orc_cfg *cfg, const orc_model_full *m, const orc_genome *el, int ne,
                    int cpu_threads, orc_survivor *out, uint64_t out_cap, uint64_t *n_out,
                    uint64_t *screened);

/* Candidate-start walk: number of candidates of stream t that start before
 * draw position `end`, starting from the candidate at draw `start`. */
uint64_t orc_walk(const orc_cfg *cfg, uint64_t t, uint64_t start, uint64_t end,
                  uint64_t *first_at_or_after_end);

#ifdef __cplusplus
}
#endif
#endif
