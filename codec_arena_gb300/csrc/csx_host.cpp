// csx_host.cpp — host side of the screen C ABI: model / genome text I/O,
// survivor formatting and the `arena screen` verb. No device code here; the
// GPU entry points live in csx_screen.cu.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/csx_screen.h"

namespace {

bool valid_n(int n) {
    return n == 153 || n == 159 || n == 161 || n == 164 || n == 165 || n == 166;
}

// std.fmt.parseInt(uN, tok, 10): optional '+', '-' only for zero, '_' allowed
// between digits.
bool parse_uint(const char *s, size_t n, uint64_t max, uint64_t *out) {
    if (n == 0) return false;
    bool neg = false;
    if (s[0] == '+' || s[0] == '-') {
        neg = s[0] == '-';
        ++s;
        --n;
    }
    if (n == 0 || s[0] == '_' || s[n - 1] == '_') return false;
    uint64_t x = 0;
    for (size_t i = 0; i < n; ++i) {
        const char c = s[i];
        if (c == '_') continue;
        if (c < '0' || c > '9') return false;
        const uint64_t d = static_cast<uint64_t>(c - '0');
        if (x > (max - d) / 10) return false;
        x = x * 10 + d;
    }
    if (neg && x != 0) return false;
    *out = x;
    return true;
}

bool is_hexdigit(char c) {
    return (c >= '0' && c <= '9') || (c >= 'a' && c <= 'f') || (c >= 'A' && c <= 'F');
}

// std.fmt.parseFloat(f32, tok): a correctly rounded decimal (or hex) -> f32
// conversion of the whole token; '_' separators between digits are dropped.
bool parse_f32(const char *s, size_t n, float *out) {
    char buf[160];
    size_t k = 0;
    if (n == 0 || n >= sizeof(buf)) return false;
    for (size_t i = 0; i < n; ++i) {
        const char c = s[i];
        if (c == '_') {
            if (i == 0 || i + 1 >= n || !is_hexdigit(s[i - 1]) || !is_hexdigit(s[i + 1]))
                return false;
            continue;
        }
        buf[k++] = c;
    }
    buf[k] = 0;
    if (std::strchr(buf, '(') != nullptr || buf[0] == ' ') return false;
    char *end = nullptr;
    errno = 0;
    const float v = std::strtof(buf, &end);
    if (end != buf + k) return false;
    *out = v;
    return true;
}

struct Tok {
    const char *p;
    size_t n;
};

bool in_set(char c, const char *set) { return c != 0 && std::strchr(set, c) != nullptr; }

// tokenizeAny: returns the count, or cap + 1 if there are more than cap.
int tokenize(const char *s, size_t len, const char *ws, Tok *toks, int cap) {
    int nt = 0;
    size_t i = 0;
    while (i < len) {
        while (i < len && in_set(s[i], ws)) ++i;
        if (i >= len) break;
        size_t j = i;
        while (j < len && !in_set(s[j], ws)) ++j;
        if (nt >= cap) return cap + 1;
        toks[nt].p = s + i;
        toks[nt].n = j - i;
        ++nt;
        i = j;
    }
    return nt;
}

bool read_file(const char *path, size_t limit, std::string *out) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::string s;
    char chunk[1 << 16];
    size_t r;
    while ((r = std::fread(chunk, 1, sizeof(chunk), f)) > 0) {
        s.append(chunk, r);
        if (s.size() > limit) {
            std::fclose(f);
            return false;
        }
    }
    const bool ok = !std::ferror(f);
    std::fclose(f);
    *out = std::move(s);
    return ok;
}

int fmt4(char *buf, size_t cap, float x) { return std::snprintf(buf, cap, "%.4f", static_cast<double>(x)); }

}  // namespace

extern "C" {

int csx_abi_version(void) { return CSX_ABI_VERSION; }

const char *csx_strerror(int status) {
    switch (status) {
        case CSX_OK: return "ok";
        case CSX_ERR_BAD_MODEL: return "BadModel";
        case CSX_ERR_NEED_TWO_ELITES: return "NeedTwoElites";
        case CSX_ERR_BAD_ARGS: return "BadArgs";
        case CSX_ERR_PARSE: return "InvalidCharacter";
        case CSX_ERR_IO: return "FileError";
        case CSX_ERR_LIMIT: return "LimitExceeded";
        case CSX_ERR_CUDA: return "CudaError";
        case CSX_ERR_NO_DEVICE: return "NoCudaDevice";
        case CSX_ERR_OOM: return "OutOfMemory";
        case CSX_ERR_DEVICE_STATE: return "DeviceErrorFlag";
        default: return "UnknownError";
    }
}

void csx_cfg_default(csx_cfg *cfg) {
    // src/main.zig:161 (lambda, keep, seed) and src/screen.zig:133-136
    cfg->lambda = 1000000;
    cfg->keep = 192;
    cfg->seed = 42;
    cfg->threads = 4;
    cfg->sigma = 0.12f;
    cfg->jump_p = 0.02f;
    cfg->imm_p = 0.01f;
    cfg->flags = 0;
}

// Model.fromCompact: src/screen.zig:36-95.
int csx_model_from_compact(const float *w, int n, csx_model *m) {
    if (!w || !m) return CSX_ERR_BAD_ARGS;
    if (!valid_n(n)) return CSX_ERR_BAD_MODEL;
    std::memset(m, 0, sizeof(*m));
    m->w0 = w[0];
    for (int i = 0; i < 16; ++i) m->w_lin[i] = w[1 + i];
    if (n == 166) {  // + intra_pred deblock entropy cfl cdef qpel sb16, then regs
        for (int i = 0; i < 7; ++i) m->w_lin[16 + i] = w[17 + i];
        for (int i = 0; i < CSX_NR; ++i) m->w_lin[CSX_NG + i] = w[24 + i];
    } else if (n == 165) {
        for (int i = 0; i < 6; ++i) m->w_lin[16 + i] = w[17 + i];
        for (int i = 0; i < CSX_NR; ++i) m->w_lin[CSX_NG + i] = w[23 + i];
    } else if (n == 164) {
        for (int i = 0; i < 5; ++i) m->w_lin[16 + i] = w[17 + i];
        for (int i = 0; i < CSX_NR; ++i) m->w_lin[CSX_NG + i] = w[22 + i];
    } else if (n == 161) {
        m->w_lin[16] = w[17];
        m->w_lin[17] = w[18];
        for (int i = 0; i < CSX_NR; ++i) m->w_lin[CSX_NG + i] = w[19 + i];
    } else if (n == 159) {
        for (int i = 0; i < CSX_NR; ++i) m->w_lin[16 + i] = w[17 + i];
    }
    int idx = n == 153 ? 17 : n == 159 ? 23 : n == 161 ? 25 : n == 164 ? 28 : n == 165 ? 29 : 30;
    for (int i = 0; i < 16; ++i)
        for (int j = 0; j <= i; ++j) m->w_quad[i * 16 + j] = w[idx++];
    return CSX_OK;
}

// loadModel body: src/screen.zig:118-126.
namespace {
// loadModel's text body; allow_full also takes the full surface's 465
// coefficients (the `arena screen` verb of this implementation).
int model_parse(const char *txt, size_t len, float *w, int cap, int *n_out, bool allow_full) {
    if (!txt || !w || !n_out) return CSX_ERR_BAD_ARGS;
    const char *ws = " \t\r\n";
    size_t i = 0;
    auto next_tok = [&](Tok *t) -> bool {
        while (i < len && in_set(txt[i], ws)) ++i;
        if (i >= len) return false;
        size_t j = i;
        while (j < len && !in_set(txt[j], ws)) ++j;
        t->p = txt + i;
        t->n = j - i;
        i = j;
        return true;
    };
    Tok t;
    if (!next_tok(&t)) return CSX_ERR_BAD_MODEL;
    uint64_t n64;
    if (!parse_uint(t.p, t.n, UINT64_MAX, &n64)) return CSX_ERR_PARSE;
    if (n64 > 1000 || !(valid_n(static_cast<int>(n64)) || (allow_full && n64 == CSX_FULL_NF)))
        return CSX_ERR_BAD_MODEL;
    const int n = static_cast<int>(n64);
    if (n > cap) return CSX_ERR_BAD_ARGS;
    for (int k = 0; k < n; ++k) {
        if (!next_tok(&t)) return CSX_ERR_BAD_MODEL;
        if (!parse_f32(t.p, t.n, &w[k])) return CSX_ERR_PARSE;
    }
    *n_out = n;
    return CSX_OK;
}
}  // namespace

int csx_model_parse(const char *txt, size_t len, float *w, int cap, int *n_out) {
    return model_parse(txt, len, w, cap, n_out, false);
}

// parseLine: src/genome.zig:116-188.
int csx_genome_parse_line(const char *line, size_t len, uint32_t flags, csx_genome *out) {
    if (!line || !out) return CSX_ERR_BAD_ARGS;
    Tok tok[35];
    const int n = tokenize(line, len, " \t\r", tok, 34);
    if (n > 34) return CSX_ERR_PARSE;  // error.BadLine
    if (!(n == 21 || n == 27 || n == 29 || n == 32 || n == 33 || n == 34)) return 0;
    if (tok[0].n > 0 && tok[0].p[0] == '#') return 0;
    csx_genome g;
    std::memset(&g, 0, sizeof(g));
    uint64_t v;
    if (!parse_uint(tok[0].p, tok[0].n, UINT64_MAX, &v)) return CSX_ERR_PARSE;
    g.id = v;
    if (!parse_uint(tok[1].p, tok[1].n, UINT32_MAX, &v)) return CSX_ERR_PARSE;
    g.gen = static_cast<uint32_t>(v);
    if (!parse_uint(tok[2].p, tok[2].n, UINT64_MAX, &v)) return CSX_ERR_PARSE;
    g.pa = v;
    if (!parse_uint(tok[3].p, tok[3].n, UINT64_MAX, &v)) return CSX_ERR_PARSE;
    g.pb = v;
    if (!parse_uint(tok[4].p, tok[4].n, UINT32_MAX, &v)) return CSX_ERR_PARSE;
    g.tribe = static_cast<uint32_t>(v);
    auto pf = [&](int gi, int ti) { return parse_f32(tok[ti].p, tok[ti].n, &g.g[gi]); };
    for (int i = 0; i < 16; ++i)
        if (!pf(i, 5 + i)) return CSX_ERR_PARSE;
    // As written, a 34-token line matches none of the v0.4/v0.5/v0.5b branches
    // and keeps g[16..21] = 0.0 (NEW_GENE_LEGACY); CSX_FLAG_PARSE_V6_FIX reads them.
    const bool fix = (flags & CSX_FLAG_PARSE_V6_FIX) != 0;
    if (n == 29 || n == 32 || n == 33 || (fix && n == 34)) {
        if (!pf(16, 21) || !pf(17, 22)) return CSX_ERR_PARSE;
    }
    if (n == 32 || n == 33 || (fix && n == 34)) {
        if (!pf(18, 23) || !pf(19, 24) || !pf(20, 25)) return CSX_ERR_PARSE;
    }
    if (n == 33 || (fix && n == 34)) {
        if (!pf(21, 26)) return CSX_ERR_PARSE;
    }
    if (n == 34) {
        if (!pf(22, 27)) return CSX_ERR_PARSE;
    }
    const int reg0 = n == 27 ? 21 : n == 29 ? 23 : n == 32 ? 26 : n == 33 ? 27 : n == 34 ? 28 : -1;
    for (int i = 0; i < CSX_NR; ++i) {
        if (reg0 < 0) {
            g.g[CSX_NG + i] = 0.5f;  // v1 line: neutral regulators
        } else if (!pf(CSX_NG + i, reg0 + i)) {
            return CSX_ERR_PARSE;
        }
    }
    *out = g;
    return 1;
}

// The elites loop of src/main.zig:201-214.
int csx_elites_parse(const char *txt, size_t len, uint32_t flags, csx_genome *out, int cap,
                     int *n_out) {
    if (!txt || !n_out || (cap > 0 && !out)) return CSX_ERR_BAD_ARGS;
    int ne = 0;
    size_t i = 0;
    while (i < len) {
        while (i < len && txt[i] == '\n') ++i;
        if (i >= len) break;
        size_t j = i;
        while (j < len && txt[j] != '\n') ++j;
        size_t a = i, b = j;
        while (a < b && in_set(txt[a], " \t\r")) ++a;
        while (b > a && in_set(txt[b - 1], " \t\r")) --b;
        i = j;
        if (a == b || txt[a] == '#') continue;
        csx_genome g;
        if (csx_genome_parse_line(txt + a, b - a, flags, &g) <= 0) continue;
        if (ne < cap) out[ne] = g;
        ++ne;
    }
    *n_out = ne;
    return CSX_OK;
}

// formatLine: src/genome.zig:191-201.
int csx_genome_format_line(const csx_genome *g, char *buf, size_t cap) {
    if (!g || !buf) return CSX_ERR_BAD_ARGS;
    size_t k = 0;
    int r = std::snprintf(buf, cap, "%llu %u %llu %llu %u", static_cast<unsigned long long>(g->id),
                          g->gen, static_cast<unsigned long long>(g->pa),
                          static_cast<unsigned long long>(g->pb), g->tribe);
    if (r < 0 || static_cast<size_t>(r) >= cap) return CSX_ERR_LIMIT;
    k = static_cast<size_t>(r);
    for (int i = 0; i < CSX_NTOT; ++i) {
        if (k + 1 >= cap) return CSX_ERR_LIMIT;
        buf[k++] = ' ';
        r = fmt4(buf + k, cap - k, g->g[i]);
        if (r < 0 || static_cast<size_t>(r) >= cap - k) return CSX_ERR_LIMIT;
        k += static_cast<size_t>(r);
    }
    return static_cast<int>(k);
}

// A promoted line. src/screen.zig:327-336 writes "0 0 pa pb tribe" and genes
// 0..23 only (29 tokens); the default here writes all 29 genes (34 tokens), the
// width brain/evolve.py:449 accepts.
int csx_survivor_format_line(const csx_survivor *s, uint32_t flags, char *buf, size_t cap) {
    if (!s || !buf) return CSX_ERR_BAD_ARGS;
    const int ng = (flags & CSX_FLAG_OUTPUT_29) ? 24 : CSX_NTOT;
    int r = std::snprintf(buf, cap, "0 0 %llu %llu %u", static_cast<unsigned long long>(s->pa),
                          static_cast<unsigned long long>(s->pb), s->tribe);
    if (r < 0 || static_cast<size_t>(r) >= cap) return CSX_ERR_LIMIT;
    size_t k = static_cast<size_t>(r);
    for (int i = 0; i < ng; ++i) {
        if (k + 1 >= cap) return CSX_ERR_LIMIT;
        buf[k++] = ' ';
        r = fmt4(buf + k, cap - k, s->g[i]);
        if (r < 0 || static_cast<size_t>(r) >= cap - k) return CSX_ERR_LIMIT;
        k += static_cast<size_t>(r);
    }
    if (k + 2 > cap) return CSX_ERR_LIMIT;
    buf[k++] = '\n';
    buf[k] = 0;
    return static_cast<int>(k);
}

// `arena screen`: flag parsing of src/main.zig:156-200, model and elites
// loading (:201-214), run() and its file output (src/screen.zig:257-343).
int csx_screen_cli(int argc, const char *const *argv) {
    std::string model_path = "state/surrogate.txt";
    std::string elites_path = "out/elites.txt";
    std::string out_path = "out/promoted.txt";
    std::string count_out = "out/screens.txt";
    csx_cfg cfg;
    csx_cfg_default(&cfg);
    auto fail = [](int st, const char *what) {
        std::fprintf(stderr, "error: %s%s%s\n", csx_strerror(st), what ? ": " : "", what ? what : "");
        return st;
    };
    auto is_switch = [](const char *a) {
        return !std::strcmp(a, "--compat-29") || !std::strcmp(a, "--as-shipped") ||
               !std::strcmp(a, "--parse-v6-fix") || !std::strcmp(a, "--exact-all");
    };
    for (int i = 0; i < argc; ++i) {
        const char *a = argv[i];
        // a trailing flag without its value is BadArgs (src/main.zig:166)
        if (i + 1 >= argc && a[0] == '-' && !is_switch(a)) return fail(CSX_ERR_BAD_ARGS, a);
        auto val = [&]() -> const char * { return argv[++i]; };
        auto u64 = [&](uint64_t *dst) -> bool {
            const char *v = val();
            return parse_uint(v, std::strlen(v), UINT64_MAX, dst);
        };
        auto f32 = [&](float *dst) -> bool {
            const char *v = val();
            return parse_f32(v, std::strlen(v), dst);
        };
        bool ok = true;
        if (!std::strcmp(a, "--model")) model_path = val();
        else if (!std::strcmp(a, "--elites")) elites_path = val();
        else if (!std::strcmp(a, "--out")) out_path = val();
        else if (!std::strcmp(a, "--count-out")) count_out = val();
        else if (!std::strcmp(a, "--lambda")) ok = u64(&cfg.lambda);
        else if (!std::strcmp(a, "--keep")) ok = u64(&cfg.keep);
        else if (!std::strcmp(a, "--seed")) ok = u64(&cfg.seed);
        else if (!std::strcmp(a, "--threads")) ok = u64(&cfg.threads);
        else if (!std::strcmp(a, "--sigma")) ok = f32(&cfg.sigma);
        else if (!std::strcmp(a, "--jump")) ok = f32(&cfg.jump_p);
        else if (!std::strcmp(a, "--imm")) ok = f32(&cfg.imm_p);
        // options of this implementation (no reference counterpart)
        else if (!std::strcmp(a, "--compat-29")) cfg.flags |= CSX_FLAG_OUTPUT_29;
        else if (!std::strcmp(a, "--as-shipped")) cfg.flags |= CSX_FLAG_AS_SHIPPED;
        else if (!std::strcmp(a, "--parse-v6-fix")) cfg.flags |= CSX_FLAG_PARSE_V6_FIX;
        else if (!std::strcmp(a, "--exact-all")) cfg.flags |= CSX_FLAG_EXACT_ALL;
        if (!ok) return fail(CSX_ERR_PARSE, a);
    }
    std::string txt;
    if (!read_file(model_path.c_str(), 1u << 20, &txt)) return fail(CSX_ERR_IO, model_path.c_str());
    // a model file of 465 coefficients is the full 29-gene surface (an
    // extension: the reference's loadModel refuses it)
    std::vector<float> w(CSX_FULL_NF);
    int n = 0;
    int st = model_parse(txt.data(), txt.size(), w.data(), CSX_FULL_NF, &n, true);
    if (st) return fail(st, model_path.c_str());
    const bool full = n == CSX_FULL_NF;
    csx_model model{};
    csx_model_full model_full{};
    st = full ? csx_model_full_from_compact(w.data(), n, &model_full) : csx_model_from_compact(w.data(), n, &model);
    if (st) return fail(st, model_path.c_str());
    if (!read_file(elites_path.c_str(), 1u << 22, &txt)) return fail(CSX_ERR_IO, elites_path.c_str());
    int ne = 0;
    csx_elites_parse(txt.data(), txt.size(), cfg.flags, nullptr, 0, &ne);
    std::vector<csx_genome> elites(static_cast<size_t>(ne > 0 ? ne : 1));
    csx_elites_parse(txt.data(), txt.size(), cfg.flags, elites.data(), ne, &ne);
    if (ne < 2) return fail(CSX_ERR_NEED_TWO_ELITES, nullptr);
    const uint64_t cap = cfg.keep < cfg.lambda ? cfg.keep : cfg.lambda;
    std::vector<csx_survivor> surv(static_cast<size_t>(cap > 0 ? cap : 1));
    uint64_t n_out = 0, screened = 0;
    st = full ? csx_screen_full(&cfg, &model_full, elites.data(), ne, surv.data(), cap, &n_out, &screened)
              : csx_screen(&cfg, &model, elites.data(), ne, surv.data(), cap, &n_out, &screened);
    if (st) return fail(st, nullptr);
    FILE *f = std::fopen(out_path.c_str(), "wb");
    if (!f) return fail(CSX_ERR_IO, out_path.c_str());
    char line[1024];
    for (uint64_t q = 0; q < n_out; ++q) {
        const int len = csx_survivor_format_line(&surv[q], cfg.flags, line, sizeof(line));
        if (len < 0 || std::fwrite(line, 1, static_cast<size_t>(len), f) != static_cast<size_t>(len)) {
            std::fclose(f);
            return fail(CSX_ERR_IO, out_path.c_str());
        }
    }
    if (std::fclose(f)) return fail(CSX_ERR_IO, out_path.c_str());
    f = std::fopen(count_out.c_str(), "wb");
    if (!f) return fail(CSX_ERR_IO, count_out.c_str());
    std::fprintf(f, "%llu\n", static_cast<unsigned long long>(screened));
    if (std::fclose(f)) return fail(CSX_ERR_IO, count_out.c_str());
    std::fprintf(stderr, "screen: %llu candidates scored, top %llu promoted\n",
                 static_cast<unsigned long long>(screened), static_cast<unsigned long long>(cfg.keep));
    return CSX_OK;
}

}  // extern "C"
