/*
 * csx_screen.h — C ABI of the GB300 screen funnel (libcsx_screen.so).
 *
 * The reference exposes its screen as a process boundary: the `arena screen`
 * verb (src/main.zig:98-101,156-218) reads a surrogate file and an elites
 * file, runs src/screen.zig:run and writes the promoted survivors and the
 * candidate count. This header is the in-process replacement for that
 * boundary: plain pointers and sizes, integer status codes, no exceptions and
 * no C++ or torch types. Every entry point names the reference symbol it
 * replaces.
 *
 * Threading: every call is synchronous unless it takes a `cuda_stream`
 * argument. Calls may come from several host threads; device scratch is kept
 * per device and guarded by a lock.
 */
#ifndef CSX_SCREEN_H
#define CSX_SCREEN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CSX_ABI_VERSION 1

#define CSX_NG 23   /* effector genes   (src/genome.zig:14) */
#define CSX_NR 6    /* regulator genes  (src/genome.zig:15) */
#define CSX_NTOT 29 /* flat genome size (src/genome.zig:16) */

/* Status codes. The first three mirror the Zig errors of the screen path. */
enum {
    CSX_OK = 0,
    CSX_ERR_BAD_MODEL = -1,       /* error.BadModel       src/screen.zig:37,120 */
    CSX_ERR_NEED_TWO_ELITES = -2, /* error.NeedTwoElites  src/screen.zig:266, src/main.zig:214 */
    CSX_ERR_BAD_ARGS = -3,        /* error.BadArgs        src/main.zig:166 */
    CSX_ERR_PARSE = -4,           /* std.fmt.parseInt / parseFloat failure */
    CSX_ERR_IO = -5,              /* file open / read / write failure */
    CSX_ERR_LIMIT = -6,           /* size beyond this build's device limits */
    CSX_ERR_CUDA = -7,            /* a CUDA runtime call failed */
    CSX_ERR_NO_DEVICE = -8,       /* no CUDA device visible */
    CSX_ERR_OOM = -9,             /* host or device allocation failed */
    CSX_ERR_DEVICE_STATE = -10    /* a kernel raised its error flag */
};

/* Flags for csx_cfg.flags and the parse / format calls. */
#define CSX_FLAG_AS_SHIPPED 0x1u   /* write no survivors, as the shipped binary does
                                      (src/screen.zig:221,285,309-313) */
#define CSX_FLAG_OUTPUT_29 0x2u    /* survivor lines in the reference's 29-token form
                                      (src/screen.zig:327-336); default is the 34-token
                                      v6 pop line (src/genome.zig:191-201) */
#define CSX_FLAG_PARSE_V6_FIX 0x4u /* 34-token elite lines keep genes 16..21; as written
                                      the reference sets them to 0.0 (src/genome.zig:138-158) */
#define CSX_FLAG_EXACT_ALL 0x8u    /* score every candidate in the reference's f32 order
                                      instead of filtering with a certified fast score */
#define CSX_FLAG_STAGE_TIMES 0x10u /* record per-stage device times (csx_last_run_info) */
#define CSX_FLAG_TC_BF16 0x20u     /* precision form: survivors ranked by their FP64 score (rounded
                                      to f32): the FP64 top-K, genes bit-exact. By default the
                                      pruning bound runs on BF16 tensor cores and the candidates it
                                      cannot rule out are filtered by FFMA and scored in FP64; with
                                      CSX_FLAG_NO_PRUNE the quadratic block of every candidate runs
                                      on the tensor cores and candidates within max(1e-3 relative,
                                      the form's certified error bound) of the K-th score are
                                      rescored in FP64. csx_screen / csx_screen_device */
#define CSX_FLAG_TC_FP16 0x40u     /* the same with FP16 tiles (unpruned: x' = 2g - 1) */
#define CSX_FLAG_NO_PRUNE 0x80u    /* score every candidate's full synthesis (the filter form)
                                      instead of skipping, by a certified bound taken after the
                                      crossover bits, candidates that cannot reach the top-K.
                                      Results are identical either way; only speed differs.
                                      Without the flag the library prunes generations of at least
                                      400 candidates per screen thread (3 CTAs x 256 threads per
                                      SM: 4.67e7 on 152 SMs; below, the unpruned kernel is
                                      faster); the environment variable CSX_PRUNE_MIN_CANDS sets
                                      that floor in candidates */
#define CSX_FLAG_PRUNE_FFMA 0x100u /* the pruning bound's gradient by FP32 FMA instead of the
                                      tensor cores (FP16 tcgen05.mma with a certified error
                                      share). Results are identical either way */

/* Model: the flat weight layout of src/screen.zig:23-27. */
typedef struct csx_model {
    float w0;
    float w_lin[CSX_NTOT];
    float w_quad[256]; /* 16x16 over the legacy effectors, zero strict upper triangle */
} csx_model;

/* Genome: src/genome.zig:78-86, genes flattened to 23 effectors + 6 regulators
 * (the order src/screen.zig:240-241 reads them in). */
typedef struct csx_genome {
    uint64_t id;
    uint64_t pa;
    uint64_t pb;
    uint32_t gen;
    uint32_t tribe;
    float g[CSX_NTOT];
    uint32_t reserved;
} csx_genome;

/* Screen configuration: src/screen.zig:129-137 (Cfg). */
typedef struct csx_cfg {
    uint64_t lambda;  /* candidates to synthesise (the --lambda count) */
    uint64_t keep;    /* survivors to keep (K) */
    uint64_t seed;    /* base seed; stream t uses seed ^ (0x9E3779B97F4A7C15 * (t+1)) */
    uint64_t threads; /* RNG stream count T, part of the result's identity */
    float sigma;      /* mutation half-width */
    float jump_p;     /* jump probability */
    float imm_p;      /* immigrant probability */
    uint32_t flags;   /* CSX_FLAG_* */
} csx_cfg;

/* Survivor: the Slot of src/screen.zig:145-149 plus its provenance. */
typedef struct csx_survivor {
    float score;      /* Model.score in the reference's f32 op order */
    uint32_t tribe;   /* lineage tribe: the first parent's tribe */
    uint64_t pa;      /* lineage: first parent's id */
    uint64_t pb;      /* lineage: second parent's id */
    uint64_t stream;  /* RNG stream t */
    uint64_t index;   /* candidate index within stream t */
    uint64_t draw;    /* splitmix64 draw position of the candidate's first draw */
    float g[CSX_NTOT];
    uint32_t reserved;
} csx_survivor;

/* ---- library ---------------------------------------------------------- */

int csx_abi_version(void);
const char *csx_strerror(int status);
/* Defaults of src/screen.zig:129-137 and src/main.zig:161. */
void csx_cfg_default(csx_cfg *cfg);

/* ---- model and genome I/O (host) --------------------------------------- */

/* Model.fromCompact, src/screen.zig:36-95: n in {153,159,161,164,165,166}. */
int csx_model_from_compact(const float *w, int n, csx_model *out);
/* loadModel's text body, src/screen.zig:115-127: "n w0 w1 ...". */
int csx_model_parse(const char *text, size_t len, float *w, int cap, int *n_out);
/* parseLine, src/genome.zig:116-188. Returns 1 (parsed), 0 (not a genome
 * line: wrong token count or comment) or a negative status. */
int csx_genome_parse_line(const char *line, size_t len, uint32_t flags, csx_genome *out);
/* The elites loop of src/main.zig:201-214: skips blank, '#' and bad lines.
 * *n_out is the number of genomes found (may exceed cap; only cap stored). */
int csx_elites_parse(const char *text, size_t len, uint32_t flags, csx_genome *out, int cap,
                     int *n_out);
/* formatLine, src/genome.zig:191-201 (34 tokens). Returns chars written. */
int csx_genome_format_line(const csx_genome *g, char *buf, size_t cap);
/* One promoted line: src/screen.zig:327-336 with CSX_FLAG_OUTPUT_29, else the
 * 34-token v6 form with id and gen 0. Returns chars written (with '\n'). */
int csx_survivor_format_line(const csx_survivor *s, uint32_t flags, char *buf, size_t cap);

/* ---- the screen (GPU) --------------------------------------------------- */

/* run(), src/screen.zig:257-343, without the file output: host buffers in and
 * out. Writes min(keep, lambda) survivors (0 with CSX_FLAG_AS_SHIPPED) sorted
 * by score descending, then stream ascending, and exact f32 ties inside a
 * stream as the reference's per-stream heap ranks them (src/screen.zig:
 * 151-193,306-319; those streams' heaps are replayed exactly: the rare calls
 * that hold such ties take longer); *screened is the
 * candidate count the reference writes to --count-out. Synchronous. */
int csx_screen(const csx_cfg *cfg, const csx_model *model, const csx_genome *elites,
               int n_elites, csx_survivor *out, uint64_t out_cap, uint64_t *n_out,
               uint64_t *screened);

/* csx_screen restricted to the RNG streams [t_begin, t_end) of the same
 * generation (0 <= t_begin < t_end <= T, T = max(1, min(threads, lambda))):
 * one rank's share when a generation is sharded by stream across GPUs.
 * Survivors carry their global stream ids; the top-K of all ranks' survivors
 * in the order score descending, (stream, index) ascending equals csx_screen's
 * result. *screened counts the range's candidates. No reference counterpart
 * (the reference runs every stream in one process). */
int csx_screen_range(const csx_cfg *cfg, const csx_model *model, const csx_genome *elites, int n_elites,
                     uint64_t t_begin, uint64_t t_end, csx_survivor *out, uint64_t out_cap, uint64_t *n_out,
                     uint64_t *screened);

/* csx_screen restricted to one share of the generation's work items: the
 * items (runs of consecutive candidates of one stream, built from the
 * configuration alone, whatever GPU runs the call) are cut into n_shards
 * contiguous parts and this call screens part `shard` (0 <= shard <
 * n_shards). Survivors carry their global stream and index; the top-K of all
 * shards' survivors in the order score descending, (stream, index)
 * ascending equals csx_screen's result, and the shards' *screened sum to
 * lambda. This splits one generation over any number of ranks, even more
 * ranks than RNG streams (csx_screen_range splits by stream). A share may be
 * empty. No reference counterpart (the reference runs every stream in one
 * process). */
int csx_screen_items(const csx_cfg *cfg, const csx_model *model, const csx_genome *elites, int n_elites,
                     uint32_t shard, uint32_t n_shards, csx_survivor *out, uint64_t out_cap, uint64_t *n_out,
                     uint64_t *screened);

/* Same, with device-resident elites and survivors, enqueued on `cuda_stream`
 * (exact f32 ties inside one stream ranked by index: the heap replay needs
 * the host; so do csx_screen_items shares and csx_screen_batch_device)
 * (a cudaStream_t; NULL = the legacy default stream). d_result receives four
 * device uint64: survivor count, screened count, device error bits (0 = ok)
 * and the number of work items screened. The call returns after enqueueing; calls on different
 * streams are ordered after one another by the library. */
int csx_screen_device(const csx_cfg *cfg, const csx_model *model, const csx_genome *d_elites,
                      int n_elites, csx_survivor *d_out, uint64_t out_cap, uint64_t *d_result,
                      void *cuda_stream);

/* No counterpart in the reference. csx_screen_device for callers that cannot
 * allocate device memory: a process whose own memory pool owns the whole
 * device, or a caller that cannot afford the implicit device-wide
 * synchronisation of cudaMalloc / cudaFree while its other streams run. This
 * call allocates nothing: its scratch is a 32 MiB array compiled into the
 * library, which every GPU that loads the library holds until the process
 * exits. Configurations needing more scratch return CSX_ERR_LIMIT with a
 * message naming the bytes needed (the 2.65e9-candidate, T = 4, keep 256
 * generation needs about 14 MiB). The first call on a device looks up the
 * array's device address; make that first call before any stream capture.
 * All calls share the array: calls that overlap on the GPU race, so order
 * them (one stream, or events). Results equal csx_screen_device's for the
 * reference surface. Not offered here: the precision-form flags
 * (CSX_FLAG_TC_BF16 / TC_FP16 return CSX_ERR_BAD_ARGS), the full surface, and
 * csx_last_run_info (not updated by this call). The device address of the
 * array is looked up on the first call and kept: a cudaDeviceReset between
 * calls is not supported. */
int csx_screen_device_noalloc(const csx_cfg *cfg, const csx_model *model, const csx_genome *d_elites,
                              int n_elites, csx_survivor *d_out, uint64_t out_cap, uint64_t *d_result,
                              void *cuda_stream);

/* The `arena screen` verb, src/main.zig:156-218 plus run()'s file output
 * (src/screen.zig:321-342): argv holds the flags after "screen". Returns 0
 * or a negative status; a message is printed to stderr on failure. */
int csx_screen_cli(int argc, const char *const *argv);

/* Device limits of this build (for callers that want to check first). */
int csx_limits(uint64_t *max_keep, uint64_t *max_elites);

/* Shape and stage times of the last screen enqueued on the current device.
 * No reference counterpart: the reference only prints the candidate count
 * (src/main.zig:217). Stage times need CSX_FLAG_STAGE_TIMES and wait for the
 * last call to finish. */
typedef struct csx_run_info {
    uint32_t launches;      /* kernels the call enqueued */
    uint32_t screen_ctas;   /* persistent screen CTAs */
    uint64_t segments;      /* walk segments (0 when streams fit one item) */
    uint64_t seg_draws;     /* draws per walk segment */
    uint64_t item_cands;    /* candidates per work item (D) */
    uint64_t items;         /* work items the screen consumed */
    float ms_prep;          /* elite table */
    float ms_items;         /* walk, assemble, scan, emit */
    float ms_screen;        /* the persistent screen kernel */
    float ms_merge;         /* top-K merge tree */
    float ms_regen;         /* survivor regeneration */
    float ms_total;
    uint64_t exact_evals;   /* candidates scored in the reference order (filter mode) */
} csx_run_info;
int csx_last_run_info(csx_run_info *out);

/* ---- batched islands --------------------------------------------------------
 * Several independent screens ("islands": the reference's CI shards, each
 * running brain/evolve.py with its own seed, elites and surrogate,
 * .github/workflows/arena.yml:56-92) in one pipeline: every island's work
 * items are built on its own forked stream; then, when every island's
 * surrogate admits the tensor-core pruning bound and every island is above
 * the pruning floor (CSX_FLAG_NO_PRUNE), each island's pruning screen runs
 * over the whole GPU in turn, else (or when any island carries
 * CSX_FLAG_NO_PRUNE) ONE unpruned persistent screen launch consumes all
 * islands' items and keeps a top-K per island; one merge tree and one
 * regeneration launch serve all islands. Results per island equal
 * csx_screen's for that island's cfg, model and elites, exact f32 ties
 * included (csx_screen_batch; see csx_screen_device for the device call).
 *
 * Tunables do not change results, only speed (0 = automatic). */
#define CSX_MAX_ISLANDS 64
typedef struct csx_batch_tune {
    uint32_t item_cands;  /* candidates per work item, rounded down to a power of two, at least 64 */
    uint32_t seg_cands;   /* candidates per walk segment */
    uint32_t ctas_per_sm; /* persistent screen CTAs per SM (1..3) */
    uint32_t reserved;
} csx_batch_tune;

/* Per-island timing of the last batch call on this device. */
typedef struct csx_batch_info {
    uint32_t islands;
    uint32_t launches;    /* kernels in the batch pipeline */
    uint32_t screen_ctas;
    uint32_t graph_nodes; /* nodes of the captured graph (host call) */
    float ms_capture;     /* host: stream capture + instantiate/update */
    float ms_device;      /* device time of the graph launch (host call) */
} csx_batch_info;

/* Host buffers. elites: all islands' genomes back to back (island i has
 * n_elites[i]); out: island i's survivors at offset sum_{j<i} keep_j;
 * n_out / screened: one per island. The pipeline is captured into a CUDA
 * graph and launched once. */
int csx_screen_batch(int n_islands, const csx_cfg *cfgs, const csx_model *models, const csx_genome *elites,
                     const int *n_elites, const csx_batch_tune *tune, csx_survivor *out, uint64_t *n_out,
                     uint64_t *screened);

/* Device buffers (same layout; d_result holds 4 words per island: count,
 * screened, error bits, items), enqueued on `cuda_stream` without a graph.
 * Not for stream capture (returns CSX_ERR_BAD_ARGS on a capturing stream):
 * its island descriptors come from a host staging area that the next batch
 * call reuses; csx_screen_batch captures and launches its own graph. */
int csx_screen_batch_device(int n_islands, const csx_cfg *cfgs, const csx_model *models,
                            const csx_genome *d_elites, const int *n_elites, const csx_batch_tune *tune,
                            csx_survivor *d_out, uint64_t *d_result, void *cuda_stream);

int csx_last_batch_info(csx_batch_info *out);

/* Model.score (src/screen.zig:97-112) of n genomes given as rows of ldg >= 29
 * device floats, in the reference's f32 operation order (the scores the screen
 * ranks by), into d_out. Asynchronous on `cuda_stream`. */
int csx_score(const csx_model *model, const float *d_genes, int64_t n, int ldg, float *d_out, void *cuda_stream);

/* ---- precision form (tensor cores) -------------------------------------------
 * No counterpart in the reference, which scores in FP32 only. The quadratic
 * block over the 16 legacy genes runs on the tensor cores (tcgen05.mma, FP32
 * accumulation in tensor memory) with the genes in BF16 (x = g) or FP16 with
 * the per-gene map x' = 2g - 1 onto [-1, 1]; constant and linear terms stay
 * FP32 on the exact genes. */
#define CSX_TC_BF16 1
#define CSX_TC_FP16 2

/* Score n genomes (rows of ldg >= 29 floats, device) in the precision form.
 * *d_err (device, zeroed by the caller) receives error bits (16: a
 * tensor-core completion wait gave up). Asynchronous on `cuda_stream`. */
int csx_tc_score(const csx_model *model, int form, const float *d_genes, int64_t n, int ldg, float *d_out,
                 uint32_t *d_err, void *cuda_stream);

/* ---- full quadratic surface -------------------------------------------------
 * No counterpart in the reference's code: docs/RESEARCH_V05C.md:99-102 queues
 * a surrogate whose quadratic block covers all 29 genes ("extend the quad
 * block in v0.6"), since the six structural genes otherwise ride linear-only.
 * Compact layout, CSX_FULL_NF = 465 floats: [0] constant, [1..29] linear
 * terms, [30..465) g_i*g_j for j <= i < 29, i outer, j inner -- the v6
 * layout's quadratic block extended from 16 to 29 genes (brain refits write
 * it; see csx_surrogate.h). Its f32 score is defined by one FMA order:
 *   r = w0; for k = 0..28: { t = w_lin[k]; for l = 0..k: t = fma(Q[k][l], g[l], t);
 *                            r = fma(g[k], t, r); }
 * i.e. w0 + sum_k g_k (w_k + sum_{l<=k} Q_kl g_l), the intercept counted
 * once. Synthesis, streams, ties, survivors and counts are csx_screen's. */
#define CSX_FULL_NF 465

typedef struct csx_model_full {
    float w0;
    float w_lin[CSX_NTOT];
    float w_quad[435]; /* (i, j <= i) at i*(i+1)/2 + j */
} csx_model_full;

/* n must be CSX_FULL_NF (else CSX_ERR_BAD_MODEL). */
int csx_model_full_from_compact(const float *w, int n, csx_model_full *out);
/* csx_screen / csx_screen_device with the candidates scored on the full
 * surface. The precision-form flags are refused (CSX_ERR_BAD_ARGS). */
int csx_screen_full(const csx_cfg *cfg, const csx_model_full *model, const csx_genome *elites, int n_elites,
                    csx_survivor *out, uint64_t out_cap, uint64_t *n_out, uint64_t *screened);
/* csx_screen_range on the full surface: the RNG streams [t_begin, t_end). */
int csx_screen_full_range(const csx_cfg *cfg, const csx_model_full *model, const csx_genome *elites,
                          int n_elites, uint64_t t_begin, uint64_t t_end, csx_survivor *out, uint64_t out_cap,
                          uint64_t *n_out, uint64_t *screened);
int csx_screen_full_device(const csx_cfg *cfg, const csx_model_full *model, const csx_genome *d_elites,
                           int n_elites, csx_survivor *d_out, uint64_t out_cap, uint64_t *d_result,
                           void *cuda_stream);
/* The full surface's score of n genomes (rows of ldg >= 29 device floats) in
 * the order above. Asynchronous on `cuda_stream`. */
int csx_score_full(const csx_model_full *model, const float *d_genes, int64_t n, int ldg, float *d_out,
                   void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* CSX_SCREEN_H */
