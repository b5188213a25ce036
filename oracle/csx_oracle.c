/*
 * csx_oracle.c — CPU restatement of codec-arena's screen funnel.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); see
 * csx_oracle.h for the list of restated reference functions and the parity
 * status. Built with -ffp-contract=off so every f32 multiply and add rounds
 * separately, as Zig's default (strict) float mode does.
 */
#include "csx_oracle.h"

#include <errno.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define GOLDEN 0x9E3779B97F4A7C15ull

/* ---- splitmix64: src/screen.zig:195-213 ---------------------------------- */

uint64_t orc_splitmix_next(uint64_t *state) {
    *state += GOLDEN;
    uint64_t z = *state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline float orc_unit(uint64_t *s) {
    /* f32(next() >> 40) * 2^-24: exact, in [0, 1) */
    return (float)(orc_splitmix_next(s) >> 40) * (1.0f / 16777216.0f);
}

/* stream seed: src/screen.zig:284 */
uint64_t orc_stream_seed(uint64_t seed, uint64_t t) { return seed ^ (GOLDEN * (t + 1)); }

/* clamp01: src/genome.zig:292-294, @max(0, @min(1, x)); NaN -> 1 (minnum). */
static inline float orc_clamp01(float x) {
    float m = (x < 1.0f) ? x : 1.0f; /* NaN compares false -> 1 */
    return (m > 0.0f) ? m : 0.0f;
}

/* ---- Model: src/screen.zig:23-112 ------------------------------------------ */

static int orc_valid_n(int n) {
    return n == 153 || n == 159 || n == 161 || n == 164 || n == 165 || n == 166;
}

int orc_model_from_compact(const float *w, int n, orc_model *m) {
    if (!orc_valid_n(n)) return ORC_ERR_BAD_MODEL;
    memset(m, 0, sizeof(*m));
    m->w0 = w[0];
    for (int i = 0; i < 16; i++) m->w_lin[i] = w[1 + i];
    /* screen.zig:45-79: the newer genes' linear slots by layout version */
    if (n == 166) {
        for (int i = 0; i < 7; i++) m->w_lin[16 + i] = w[17 + i];
        for (int i = 0; i < ORC_NR; i++) m->w_lin[ORC_NG + i] = w[24 + i];
    } else if (n == 165) {
        for (int i = 0; i < 6; i++) m->w_lin[16 + i] = w[17 + i];
        for (int i = 0; i < ORC_NR; i++) m->w_lin[ORC_NG + i] = w[23 + i];
    } else if (n == 164) {
        for (int i = 0; i < 5; i++) m->w_lin[16 + i] = w[17 + i];
        for (int i = 0; i < ORC_NR; i++) m->w_lin[ORC_NG + i] = w[22 + i];
    } else if (n == 161) {
        m->w_lin[16] = w[17];
        m->w_lin[17] = w[18];
        for (int i = 0; i < ORC_NR; i++) m->w_lin[ORC_NG + i] = w[19 + i];
    } else if (n == 159) {
        /* v2 puts the six regulator weights at flat 16..21 (screen.zig:77-79) */
        for (int i = 0; i < ORC_NR; i++) m->w_lin[16 + i] = w[17 + i];
    }
    int idx = (n == 153) ? 17 : (n == 159) ? 23 : (n == 161) ? 25 : (n == 164) ? 28
            : (n == 165) ? 29 : 30;
    for (int i = 0; i < 16; i++)
        for (int j = 0; j <= i; j++) m->w_quad[i * 16 + j] = w[idx++];
    return ORC_OK;
}

/* Model.score with the Zig vector op order: per lane l, acc = w0 + wl*g,
 * sum = sum_i (Wq[i][l] * (g[l]*g[i])) for i = 0..15, then an ordered
 * reduction of acc+sum over the 16 lanes, then + the sequential tail sum.
 * The lanes are a 16 x f32 vector as in the reference's @Vector(16, f32)
 * (GCC vector extension: NEON or SSE/AVX by target, each lane rounding its
 * own multiply and add; the build forbids contraction). */
typedef float orc_v16 __attribute__((vector_size(64)));

float orc_score(const orc_model *m, const float *g) {
    orc_v16 G, WL, acc, sum = {0};
    memcpy(&G, g, sizeof(G));
    memcpy(&WL, m->w_lin, sizeof(WL));
    acc = m->w0 + WL * G;
    for (int i = 0; i < 16; i++) {
        orc_v16 WQ;
        memcpy(&WQ, &m->w_quad[i * 16], sizeof(WQ));
        sum = sum + WQ * (G * g[i]);
    }
    const orc_v16 t = acc + sum;
    float r = -0.0f;
    for (int l = 0; l < 16; l++) r = r + t[l];
    float rsum = 0.0f;
    for (int i = 16; i < ORC_NTOT; i++) rsum = rsum + m->w_lin[i] * g[i];
    return r + rsum;
}

/* The same surface in f64. Model.score splats w0 into all 16 lanes before
 * the lane reduction (src/screen.zig:100,111), so the intercept counts 16
 * times; this restatement keeps that. */
double orc_score_f64(const orc_model *m, const float *g) {
    double s = 16.0 * (double)m->w0;
    for (int i = 0; i < ORC_NTOT; i++) s += (double)m->w_lin[i] * (double)g[i];
    for (int i = 0; i < 16; i++)
        for (int j = 0; j <= i; j++)
            s += (double)m->w_quad[i * 16 + j] * ((double)g[i] * (double)g[j]);
    return s;
}

/* ---- full quadratic surface (no reference code; see csx_oracle.h) ---------- */

int orc_model_full_from_compact(const float *w, int n, orc_model_full *m) {
    if (n != ORC_FULL_NF) return ORC_ERR_BAD_MODEL;
    m->w0 = w[0];
    for (int k = 0; k < ORC_NTOT; k++) m->w_lin[k] = w[1 + k];
    for (int q = 0; q < ORC_FULL_NQ; q++) m->w_quad[q] = w[1 + ORC_NTOT + q];
    return ORC_OK;
}

float orc_score_full(const orc_model_full *m, const float *g) {
    float r = m->w0;
    for (int k = 0; k < ORC_NTOT; k++) {
        const float *q = &m->w_quad[k * (k + 1) / 2];
        float t = m->w_lin[k];
        for (int l = 0; l <= k; l++) t = fmaf(q[l], g[l], t);
        r = fmaf(g[k], t, r);
    }
    return r;
}

double orc_score_full_f64(const orc_model_full *m, const float *g) {
    double r = (double)m->w0;
    for (int k = 0; k < ORC_NTOT; k++) {
        const float *q = &m->w_quad[k * (k + 1) / 2];
        double t = (double)m->w_lin[k];
        for (int l = 0; l <= k; l++) t += (double)q[l] * (double)g[l];
        r += (double)g[k] * t;
    }
    return r;
}

/* ---- text parsing (std.fmt.parseInt / parseFloat subset) ------------------- */

/* Zig-style unsigned parse, base 10: optional '+', '-' only for zero,
 * '_' separators allowed between digits. */
static int orc_parse_u64(const char *s, size_t n, uint64_t max, uint64_t *out) {
    if (n == 0) return -1;
    int neg = 0;
    if (s[0] == '+' || s[0] == '-') {
        neg = s[0] == '-';
        s++;
        n--;
    }
    if (n == 0 || s[0] == '_' || s[n - 1] == '_') return -1;
    uint64_t x = 0;
    for (size_t i = 0; i < n; i++) {
        char c = s[i];
        if (c == '_') continue;
        if (c < '0' || c > '9') return -1;
        uint64_t d = (uint64_t)(c - '0');
        if (x > (max - d) / 10) return -1;
        x = x * 10 + d;
    }
    if (neg && x != 0) return -1;
    *out = x;
    return 0;
}

static int orc_parse_f32(const char *s, size_t n, float *out) {
    char buf[128];
    size_t k = 0;
    if (n == 0 || n >= sizeof(buf)) return -1;
    for (size_t i = 0; i < n; i++) {
        char c = s[i];
        if (c == '_') { /* digit separator: only between two digits */
            if (i == 0 || i + 1 >= n) return -1;
            char a = s[i - 1], b = s[i + 1];
            if (!((a >= '0' && a <= '9') || (a >= 'a' && a <= 'f') || (a >= 'A' && a <= 'F')))
                return -1;
            if (!((b >= '0' && b <= '9') || (b >= 'a' && b <= 'f') || (b >= 'A' && b <= 'F')))
                return -1;
            continue;
        }
        buf[k++] = c;
    }
    buf[k] = 0;
    /* reject forms strtof accepts but Zig does not: leading space, nan(...) */
    if (buf[0] == ' ' || strchr(buf, '(')) return -1;
    char *end = NULL;
    errno = 0;
    float v = strtof(buf, &end);
    if (end != buf + k) return -1;
    *out = v;
    return 0;
}

static int is_ws(char c, const char *set) { return strchr(set, c) != NULL && c != 0; }

typedef struct { const char *p; size_t n; } tok_t;

static int tokenize(const char *s, size_t len, const char *ws, tok_t *toks, int cap) {
    int nt = 0;
    size_t i = 0;
    while (i < len) {
        while (i < len && is_ws(s[i], ws)) i++;
        if (i >= len) break;
        size_t j = i;
        while (j < len && !is_ws(s[j], ws)) j++;
        if (nt >= cap) return cap + 1;
        toks[nt].p = s + i;
        toks[nt].n = j - i;
        nt++;
        i = j;
    }
    return nt;
}

/* loadModel text body: src/screen.zig:115-127 (the file read is the caller's) */
int orc_model_parse(const char *txt, size_t len, float *w, int cap, int *n_out) {
    size_t i = 0;
    const char *ws = " \t\r\n";
    tok_t t;
    /* first token: n */
    while (i < len && is_ws(txt[i], ws)) i++;
    if (i >= len) return ORC_ERR_BAD_MODEL;
    size_t j = i;
    while (j < len && !is_ws(txt[j], ws)) j++;
    uint64_t n64;
    if (orc_parse_u64(txt + i, j - i, UINT64_MAX, &n64)) return ORC_ERR_PARSE;
    if (n64 > 1000 || !orc_valid_n((int)n64)) return ORC_ERR_BAD_MODEL;
    int n = (int)n64;
    if (n > cap) return ORC_ERR_BAD_MODEL;
    i = j;
    for (int k = 0; k < n; k++) {
        while (i < len && is_ws(txt[i], ws)) i++;
        if (i >= len) return ORC_ERR_BAD_MODEL;
        j = i;
        while (j < len && !is_ws(txt[j], ws)) j++;
        t.p = txt + i;
        t.n = j - i;
        if (orc_parse_f32(t.p, t.n, &w[k])) return ORC_ERR_PARSE;
        i = j;
    }
    *n_out = n;
    return ORC_OK;
}

/* parseLine: src/genome.zig:116-188. Returns 1 parsed, 0 skipped (wrong token
 * count / comment), <0 error. As written in the reference, a 34-token (v6)
 * line reads only g[22] of the genes beyond the legacy 16 and leaves g[16..21]
 * at 0.0; ORC_FLAG_PARSE_V6_FIX reads them from tok[21..26]. */
int orc_parse_line(const char *line, size_t len, uint32_t flags, orc_genome *out) {
    tok_t tok[35];
    int n = tokenize(line, len, " \t\r", tok, 34);
    if (n > 34) return ORC_ERR_PARSE; /* error.BadLine */
    if (!(n == 21 || n == 27 || n == 29 || n == 32 || n == 33 || n == 34)) return 0;
    if (tok[0].n > 0 && tok[0].p[0] == '#') return 0;
    orc_genome gm;
    memset(&gm, 0, sizeof(gm));
    uint64_t v;
    if (orc_parse_u64(tok[0].p, tok[0].n, UINT64_MAX, &v)) return ORC_ERR_PARSE;
    gm.id = v;
    if (orc_parse_u64(tok[1].p, tok[1].n, UINT32_MAX, &v)) return ORC_ERR_PARSE;
    gm.gen = (uint32_t)v;
    if (orc_parse_u64(tok[2].p, tok[2].n, UINT64_MAX, &v)) return ORC_ERR_PARSE;
    gm.pa = v;
    if (orc_parse_u64(tok[3].p, tok[3].n, UINT64_MAX, &v)) return ORC_ERR_PARSE;
    gm.pb = v;
    if (orc_parse_u64(tok[4].p, tok[4].n, UINT32_MAX, &v)) return ORC_ERR_PARSE;
    gm.tribe = (uint32_t)v;
#define PF(dst, ti) \
    do { if (orc_parse_f32(tok[ti].p, tok[ti].n, &(dst))) return ORC_ERR_PARSE; } while (0)
    for (int i = 0; i < 16; i++) PF(gm.g[i], 5 + i);
    const int fix = (flags & ORC_FLAG_PARSE_V6_FIX) != 0;
    if (n == 29 || n == 32 || n == 33 || (fix && n == 34)) {
        PF(gm.g[16], 21);
        PF(gm.g[17], 22);
    }
    if (n == 32 || n == 33 || (fix && n == 34)) {
        PF(gm.g[18], 23);
        PF(gm.g[19], 24);
        PF(gm.g[20], 25);
    }
    if (n == 33 || (fix && n == 34)) PF(gm.g[21], 26);
    if (n == 34) PF(gm.g[22], 27);
    int reg0 = (n == 27) ? 21 : (n == 29) ? 23 : (n == 32) ? 26 : (n == 33) ? 27 : (n == 34) ? 28 : -1;
    for (int i = 0; i < ORC_NR; i++) {
        if (reg0 < 0)
            gm.g[ORC_NG + i] = 0.5f;
        else
            PF(gm.g[ORC_NG + i], reg0 + i);
    }
#undef PF
    *out = gm;
    return 1;
}

/* elites file body: src/main.zig:201-214 */
int orc_elites_parse(const char *txt, size_t len, uint32_t flags, orc_genome *out,
                     int cap, int *n_out) {
    int ne = 0;
    size_t i = 0;
    while (i < len) {
        while (i < len && txt[i] == '\n') i++;
        if (i >= len) break;
        size_t j = i;
        while (j < len && txt[j] != '\n') j++;
        size_t a = i, b = j;
        while (a < b && (txt[a] == ' ' || txt[a] == '\t' || txt[a] == '\r')) a++;
        while (b > a && (txt[b - 1] == ' ' || txt[b - 1] == '\t' || txt[b - 1] == '\r')) b--;
        i = j;
        if (a == b || txt[a] == '#') continue;
        orc_genome g;
        int r = orc_parse_line(txt + a, b - a, flags, &g);
        if (r <= 0) continue; /* parse errors and null lines are skipped */
        if (ne < cap) out[ne] = g;
        ne++;
    }
    *n_out = ne;
    return ORC_OK;
}

/* ---- candidate synthesis: src/screen.zig:225-253 --------------------------- */

typedef struct {
    const orc_cfg *cfg;
    const orc_model *m;
    const orc_genome *el;
    int ne;
    const orc_model_full *mf; /* scores with the full surface when set */
} orc_ctx;

/* x % d for 32-bit x and 1 <= d < 2^32 without a divide (Lemire, Kaser,
 * Kurz 2019): m = floor((2^64 - 1) / d) + 1, x % d = hi64((m * x mod 2^64) * d). */
static inline uint32_t orc_fastmod(uint32_t x, uint64_t m, uint32_t d) {
    const uint64_t low = m * x;
    return (uint32_t)(((unsigned __int128)low * d) >> 64);
}

static float orc_synth(const orc_ctx *c, uint64_t *s, float *g, uint32_t *ea_i, uint32_t *eb_i) {
    const uint32_t ne = (uint32_t)c->ne;
    const uint64_t mag = ~0ull / ne + 1;
    const orc_genome *ea = &c->el[orc_fastmod((uint32_t)(orc_splitmix_next(s) >> 32), mag, ne)];
    const orc_genome *eb = &c->el[orc_fastmod((uint32_t)(orc_splitmix_next(s) >> 32), mag, ne)];
    *ea_i = (uint32_t)(ea - c->el);
    *eb_i = (uint32_t)(eb - c->el);
    if (orc_unit(s) < c->cfg->imm_p) {
        for (int k = 0; k < ORC_NTOT; k++) g[k] = orc_unit(s);
    } else {
        const float sigma = c->cfg->sigma;
        const float *pa = ea->g, *pb = eb->g;
        for (int k = 0; k < ORC_NTOT; k++) {
            float v = (orc_splitmix_next(s) & 1) ? pb[k] : pa[k];
            v = v + ((orc_unit(s) - 0.5f) * 2.0f) * sigma;
            g[k] = orc_clamp01(v);
        }
    }
    if (orc_unit(s) < c->cfg->jump_p) {
        /* g[idx()] = unit(): the index draw precedes the value draw */
        const uint64_t idx = (orc_splitmix_next(s) >> 32) % ORC_NTOT;
        g[idx] = orc_unit(s);
    }
    return c->mf ? orc_score_full(c->mf, g) : orc_score(c->m, g);
}

static void candidate_ctx(const orc_ctx *c, uint64_t t, uint64_t draw, orc_survivor *out,
                          uint64_t *next_draw) {
    const orc_genome *el = c->el;
    const uint64_t seed_t = orc_stream_seed(c->cfg->seed, t);
    uint64_t s = seed_t + draw * GOLDEN;
    uint32_t a, b;
    memset(out, 0, sizeof(*out));
    out->score = orc_synth(c, &s, out->g, &a, &b);
    out->pa = el[a].id;
    out->pb = el[b].id;
    out->tribe = el[a].tribe;
    out->stream = t;
    out->draw = draw;
    if (next_draw) *next_draw = (s - seed_t) * 0xF1DE83E19937733Dull; /* s = seed + d*G, G^-1 */
}

void orc_candidate(const orc_cfg *cfg, const orc_model *m, const orc_genome *el, int ne,
                   uint64_t t, uint64_t draw, orc_survivor *out, uint64_t *next_draw) {
    const orc_ctx c = {cfg, m, el, ne, NULL};
    candidate_ctx(&c, t, draw, out, next_draw);
}

void orc_candidate_full(const orc_cfg *cfg, const orc_model_full *m, const orc_genome *el, int ne,
                        uint64_t t, uint64_t draw, orc_survivor *out, uint64_t *next_draw) {
    const orc_ctx c = {cfg, NULL, el, ne, m};
    candidate_ctx(&c, t, draw, out, next_draw);
}

int orc_stream_dump(const orc_cfg *cfg, const orc_model *m, const orc_genome *el, int ne,
                    uint64_t t, uint64_t n, orc_survivor *out) {
    uint64_t d = 0;
    for (uint64_t i = 0; i < n; i++) {
        orc_candidate(cfg, m, el, ne, t, d, &out[i], &d);
        out[i].index = i;
    }
    return ORC_OK;
}

uint64_t orc_walk(const orc_cfg *cfg, uint64_t t, uint64_t start, uint64_t end,
                  uint64_t *first_at_or_after_end) {
    const uint64_t seed_t = orc_stream_seed(cfg->seed, t);
    uint64_t p = start, n = 0;
    while (p < end) {
        uint64_t s = seed_t + (p + 2) * GOLDEN;
        int imm = orc_unit(&s) < cfg->imm_p;
        uint64_t jpos = p + 3 + (imm ? 29 : 58);
        s = seed_t + jpos * GOLDEN;
        int jump = orc_unit(&s) < cfg->jump_p;
        p = jpos + 1 + (jump ? 2 : 0);
        n++;
    }
    if (first_at_or_after_end) *first_at_or_after_end = p;
    return n;
}

/* ---- heap: src/screen.zig:151-193 ------------------------------------------ */

typedef struct {
    float score;
    uint32_t pad_;
    uint64_t draw;
    uint64_t index;
} orc_slot;

static void heap_offer(orc_slot *h, uint64_t k, uint64_t *n, orc_slot s) {
    if (*n < k) {
        h[*n] = s;
        uint64_t i = *n;
        (*n)++;
        while (i > 0) {
            uint64_t parent = (i - 1) / 2;
            if (h[parent].score <= h[i].score) break;
            orc_slot tmp = h[parent];
            h[parent] = h[i];
            h[i] = tmp;
            i = parent;
        }
        return;
    }
    if (s.score <= h[0].score) return;
    h[0] = s;
    uint64_t i = 0;
    for (;;) {
        uint64_t l = 2 * i + 1, r = 2 * i + 2, mm = i;
        if (l < k && h[l].score < h[mm].score) mm = l;
        if (r < k && h[r].score < h[mm].score) mm = r;
        if (mm == i) break;
        orc_slot tmp = h[mm];
        h[mm] = h[i];
        h[i] = tmp;
        i = mm;
    }
}

/* ---- merge order: stable sort by score desc of the stream-ordered concat ---- */

typedef struct {
    float score;
    uint32_t okey;
    uint64_t stream;
    uint64_t slotpos;
    uint64_t draw;
    uint64_t index;
} orc_entry;

static uint32_t orc_okey(float x) {
    if (x != x) return 0; /* NaN ranks below every number */
    x = x + 0.0f;         /* -0 -> +0: the reference compares them equal */
    uint32_t b;
    memcpy(&b, &x, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

/* a ranks before b in the final list */
static int entry_before(const orc_entry *a, const orc_entry *b) {
    if (a->okey != b->okey) return a->okey > b->okey;
    if (a->stream != b->stream) return a->stream < b->stream;
    return a->slotpos < b->slotpos;
}

static int entry_cmp(const void *pa, const void *pb) {
    const orc_entry *a = (const orc_entry *)pa, *b = (const orc_entry *)pb;
    if (entry_before(a, b)) return -1;
    if (entry_before(b, a)) return 1;
    return 0;
}

typedef struct {
    orc_entry *v;
    uint64_t n, cap, keep;
    int have_worst;
    orc_entry worst;
} best_list;

static void best_trim(best_list *bl) {
    qsort(bl->v, bl->n, sizeof(orc_entry), entry_cmp);
    if (bl->n > bl->keep) bl->n = bl->keep;
    if (bl->n == bl->keep) {
        bl->worst = bl->v[bl->n - 1];
        bl->have_worst = 1;
    }
}

static void best_add(best_list *bl, const orc_entry *e) {
    if (bl->have_worst && !entry_before(e, &bl->worst)) return;
    bl->v[bl->n++] = *e;
    if (bl->n == bl->cap) best_trim(bl);
}

/* ---- run(): src/screen.zig:257-343 ----------------------------------------- */

typedef struct {
    orc_ctx c;
    uint64_t T, per, keep;
    uint64_t next_stream; /* shared, atomically advanced */
    pthread_mutex_t mu;
    best_list *lists;
    int nworkers;
    uint64_t screens;
    int failed;
} orc_run;

typedef struct {
    orc_run *r;
    int w;
} orc_worker_arg;

static void *orc_worker(void *arg) {
    orc_worker_arg *wa = (orc_worker_arg *)arg;
    orc_run *r = wa->r;
    best_list *bl = &r->lists[wa->w];
    orc_slot *heap = (orc_slot *)malloc(sizeof(orc_slot) * (size_t)r->keep);
    if (!heap) {
        r->failed = 1;
        return NULL;
    }
    uint64_t screens = 0;
    float g[ORC_NTOT];
    for (;;) {
        uint64_t t = __atomic_fetch_add(&r->next_stream, 1, __ATOMIC_RELAXED);
        if (t >= r->T) break;
        const uint64_t my = (t == r->T - 1) ? r->c.cfg->lambda - (r->T - 1) * r->per : r->per;
        const uint64_t seed_t = orc_stream_seed(r->c.cfg->seed, t);
        uint64_t s = seed_t, n = 0;
        for (uint64_t i = 0; i < my; i++) {
            const uint64_t draw = (s - seed_t) * 0xF1DE83E19937733Dull;
            uint32_t a, b;
            orc_slot sl;
            sl.score = orc_synth(&r->c, &s, g, &a, &b);
            sl.pad_ = 0;
            sl.draw = draw;
            sl.index = i;
            heap_offer(heap, r->keep, &n, sl);
        }
        screens += my;
        for (uint64_t q = 0; q < n; q++) {
            orc_entry e;
            e.score = heap[q].score;
            e.okey = orc_okey(heap[q].score);
            e.stream = t;
            e.slotpos = q;
            e.draw = heap[q].draw;
            e.index = heap[q].index;
            best_add(bl, &e);
        }
    }
    free(heap);
    pthread_mutex_lock(&r->mu);
    r->screens += screens;
    pthread_mutex_unlock(&r->mu);
    return NULL;
}

static int screen_ctx(const orc_ctx *ctx, int cpu_threads, orc_survivor *out, uint64_t out_cap,
                      uint64_t *n_out, uint64_t *screened) {
    const orc_cfg *cfg = ctx->cfg;
    const int ne = ctx->ne;
    *n_out = 0;
    if (screened) *screened = 0;
    if (ne < 2) return ORC_ERR_NEED_TWO_ELITES;
    if (cfg->keep == 0) return ORC_ERR_BAD_ARGS; /* Heap.offer reads slots[0] of an empty heap */
    uint64_t T = cfg->threads < cfg->lambda ? cfg->threads : cfg->lambda;
    if (T < 1) T = 1;
    orc_run r;
    memset(&r, 0, sizeof(r));
    r.c = *ctx;
    r.T = T;
    r.per = cfg->lambda / T;
    r.keep = cfg->keep;
    pthread_mutex_init(&r.mu, NULL);
    int nw = cpu_threads > 0 ? cpu_threads : (T < 64 ? (int)T : 64);
    if ((uint64_t)nw > T) nw = (int)T;
    r.nworkers = nw;
    r.lists = (best_list *)calloc((size_t)nw, sizeof(best_list));
    pthread_t *th = (pthread_t *)calloc((size_t)nw, sizeof(pthread_t));
    orc_worker_arg *args = (orc_worker_arg *)calloc((size_t)nw, sizeof(orc_worker_arg));
    int rc = ORC_OK;
    if (!r.lists || !th || !args) {
        rc = ORC_ERR_OOM;
        goto done;
    }
    for (int w = 0; w < nw; w++) {
        r.lists[w].keep = cfg->keep;
        r.lists[w].cap = 2 * cfg->keep + 1;
        r.lists[w].v = (orc_entry *)malloc(sizeof(orc_entry) * (size_t)r.lists[w].cap);
        if (!r.lists[w].v) {
            rc = ORC_ERR_OOM;
            goto done;
        }
        args[w].r = &r;
        args[w].w = w;
    }
    for (int w = 1; w < nw; w++)
        if (pthread_create(&th[w], NULL, orc_worker, &args[w])) th[w] = 0;
    orc_worker(&args[0]);
    for (int w = 1; w < nw; w++) {
        if (th[w]) pthread_join(th[w], NULL);
        else orc_worker(&args[w]);
    }
    if (r.failed) {
        rc = ORC_ERR_OOM;
        goto done;
    }
    {
        uint64_t tot = 0;
        for (int w = 0; w < nw; w++) tot += r.lists[w].n;
        orc_entry *all = (orc_entry *)malloc(sizeof(orc_entry) * (size_t)(tot ? tot : 1));
        if (!all) {
            rc = ORC_ERR_OOM;
            goto done;
        }
        uint64_t k = 0;
        for (int w = 0; w < nw; w++)
            for (uint64_t q = 0; q < r.lists[w].n; q++) all[k++] = r.lists[w].v[q];
        qsort(all, tot, sizeof(orc_entry), entry_cmp);
        uint64_t outn = tot < cfg->keep ? tot : cfg->keep;
        if (cfg->flags & ORC_FLAG_AS_SHIPPED) outn = 0;
        if (outn > out_cap) outn = out_cap;
        for (uint64_t q = 0; q < outn; q++) {
            candidate_ctx(ctx, all[q].stream, all[q].draw, &out[q], NULL);
            out[q].index = all[q].index;
        }
        *n_out = outn;
        free(all);
    }
    if (screened) *screened = r.screens;
done:
    if (r.lists)
        for (int w = 0; w < nw; w++) free(r.lists[w].v);
    free(r.lists);
    free(th);
    free(args);
    pthread_mutex_destroy(&r.mu);
    return rc;
}

int orc_screen(const orc_cfg *cfg, const orc_model *m, const orc_genome *el, int ne,
               int cpu_threads, orc_survivor *out, uint64_t out_cap, uint64_t *n_out,
               uint64_t *screened) {
    const orc_ctx c = {cfg, m, el, ne, NULL};
    return screen_ctx(&c, cpu_threads, out, out_cap, n_out, screened);
}

int orc_screen_full(const orc_cfg *cfg, const orc_model_full *m, const orc_genome *el, int ne,
                    int cpu_threads, orc_survivor *out, uint64_t out_cap, uint64_t *n_out,
                    uint64_t *screened) {
    const orc_ctx c = {cfg, NULL, el, ne, m};
    return screen_ctx(&c, cpu_threads, out, out_cap, n_out, screened);
}
