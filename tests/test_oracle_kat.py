"""The CPU oracle against the reference's own known answers (no GPU).

Pins, each citing the reference test it restates:
  * splitmix64: the published output sequence of seed 0;
  * Model.fromCompact layout: src/screen.zig:345-377;
  * Model.score monotonicity and neutrality: src/screen.zig:379-405;
  * parseLine / formatLine: src/genome.zig:296-372;
  * the surrogate refit (oracle/refit.py): outputs of brain/evolve.py's own
    features / refit_surrogate (tests/golden/evolve_golden.json).
Where a reference assertion contradicts the reference code, the test asserts
what the code computes and names the assertion it departs from.
"""
import os

import numpy as np
import pytest

from conftest import ROOT


def test_splitmix64_published_sequence(orc):
    import ctypes

    s = ctypes.c_uint64(0)
    got = [orc.lib().orc_splitmix_next(ctypes.byref(s)) for _ in range(3)]
    assert got == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_stream_seed_formula(orc):
    # src/screen.zig:284: seed ^ (0x9E3779B97F4A7C15 *% (t + 1))
    for seed, t in [(7, 0), (7, 3), (2**64 - 1, 5), (42, 1000)]:
        want = seed ^ ((0x9E3779B97F4A7C15 * (t + 1)) % 2**64)
        assert orc.lib().orc_stream_seed(seed, t) == want


def _compact(n):
    return np.arange(n, dtype=np.float32)


def test_from_compact_v1_layout(orc):
    m = orc.model_from_compact(_compact(153))
    assert m.w0 == 0 and m.w_lin[0] == 1
    assert m.w_lin[16] == 0          # regulator / newer weights neutral
    assert m.w_quad[0] == 17         # feature 17 -> (0,0)
    assert m.w_quad[16] == 18        # feature 18 -> (1,0)
    assert m.w_quad[1] == 0          # strict upper triangle
    # src/screen.zig:358 asserts 20 for quad[2*16+1], but its own comment's
    # index is 17 + T(2) + 1 = 21 and the fromCompact loop stores w[21] there.
    assert m.w_quad[33] == 21


def test_from_compact_v2_layout(orc):
    m = orc.model_from_compact(_compact(159))
    assert m.w_lin[21] == 22
    assert m.w_quad[0] == 23


def test_from_compact_v3_layout(orc):
    m = orc.model_from_compact(_compact(161))
    assert m.w_lin[16] == 17 and m.w_lin[17] == 18
    assert m.w_quad[0] == 25
    # src/screen.zig:374-375 assert w_lin[18] == 19 and w_lin[23] == 24 (an
    # older layout with the regulators right after deblock). The code puts the
    # six regulator weights at flat 23..28 (NG + i) from w[19..24].
    assert m.w_lin[18] == 0
    assert list(m.w_lin[23:29]) == [19, 20, 21, 22, 23, 24]


@pytest.mark.parametrize("n,lin_tail,reg0,quad0", [
    (164, [17, 18, 19, 20, 21, 0, 0], 22, 28),
    (165, [17, 18, 19, 20, 21, 22, 0], 23, 29),
    (166, [17, 18, 19, 20, 21, 22, 23], 24, 30),
])
def test_from_compact_v4_v6_layout(orc, n, lin_tail, reg0, quad0):
    m = orc.model_from_compact(_compact(n))
    assert list(m.w_lin[16:23]) == lin_tail
    assert list(m.w_lin[23:29]) == list(range(reg0, reg0 + 6))
    assert m.w_quad[0] == quad0
    # last quad slot (15,15) takes the last compact weight
    assert m.w_quad[255] == n - 1


def test_from_compact_rejects_other_sizes(orc):
    for n in (0, 1, 152, 154, 160, 167, 200):
        with pytest.raises(ValueError):
            orc.model_from_compact(np.zeros(max(n, 1), np.float32)[:n] if n else np.zeros(0, np.float32))


def test_score_monotone_and_neutral(orc):
    # src/screen.zig:379-405
    w = np.zeros(153, np.float32)
    w[0] = 1.0
    w[1 + 3] = 10.0
    m = orc.model_from_compact(w)
    ga = np.full(29, 0.5, np.float32)
    gb = ga.copy()
    gb[3] = 0.9
    assert orc.score(m, gb) > orc.score(m, ga)
    gc = ga.copy()
    gc[16] = 0.95
    gc[17] = 0.9
    assert orc.score(m, gc) == orc.score(m, ga)


def test_score_matches_f64_closely(orc):
    from codec_arena_gb300 import workloads as wl

    m = orc.model_from_compact(wl.surrogate_161())
    rng = np.random.default_rng(5)
    for _ in range(200):
        g = rng.random(29).astype(np.float32)
        s32 = float(orc.score(m, g))
        s64 = orc.score_f64(m, g)
        assert abs(s32 - s64) <= 1e-5 * max(1.0, abs(s64)) + 1e-3


V1 = "1 0 0 0 7 0.1 0.9 0.2 0.3 0.4 0.5 0.6 0.7 0.8 0.9 0.05 0.5 0.5 0.5 0.11 0.22"
V2 = V1.replace("1 0 0 0 7", "2 0 0 0 7") + " 0.9 0.1 0.5 0.5 0.5 0.7"


def test_parse_v1_v2(orc):
    # src/genome.zig:296-312
    g1 = orc.parse_line(V1)
    assert g1 is not None and g1["id"] == 1
    assert g1["g"][23] == np.float32(0.5) and g1["g"][28] == np.float32(0.5)  # neutral regs
    assert g1["g"][16] == 0 and g1["g"][17] == 0
    g2 = orc.parse_line(V2)
    assert g2["g"][23] == np.float32(0.9) and g2["g"][24] == np.float32(0.1)
    assert g2["g"][28] == np.float32(0.7) and g2["g"][16] == 0


def _v6_line(gen16=0.9, gen17=0.35, reg2=0.8):
    genes = [0.5] * 23
    genes[16], genes[17] = gen16, gen17
    regs = [0.5] * 6
    regs[2] = reg2
    return "77 3 9 11 5 " + " ".join(f"{x:.4f}" for x in genes + regs)


def test_parse_v6_as_written_and_fixed(orc):
    # src/genome.zig:314-331 round-trips a formatLine (34-token) line and
    # expects g[16] == 0.9. As written, parseLine's v0.4/v0.5/v0.5b branches
    # test n == 29/32/33 only, so a 34-token line reads g[16..21] as 0.0.
    line = _v6_line()
    assert len(line.split()) == 34
    g = orc.parse_line(line)
    assert g["id"] == 77 and g["g"][16] == 0.0 and g["g"][17] == 0.0
    assert g["g"][25] == np.float32(0.8)  # regulators are read
    gf = orc.parse_line(line, flags=orc.FLAG_PARSE_V6_FIX)
    assert gf["g"][16] == np.float32(0.9) and gf["g"][17] == np.float32(0.35)


def test_parse_v4_v5(orc):
    # src/genome.zig:358-372: a v4 (32-token) line migrates qpel to 0.0
    v4 = "9 1 2 3 4 " + " ".join(["0.5"] * 27)
    g4 = orc.parse_line(v4)
    assert g4["g"][21] == 0.0 and g4["g"][20] == np.float32(0.5)
    v5 = "10 2 0 0 1 " + " ".join(["0.3"] * 21 + ["0.9"] + ["0.5"] * 6)
    g5 = orc.parse_line(v5)
    assert g5["g"][21] == np.float32(0.9)


def test_parse_skips_and_errors(orc):
    assert orc.parse_line("# comment " + " ".join(["1"] * 20)) is None
    assert orc.parse_line("1 2 3") is None
    with pytest.raises(ValueError):
        orc.parse_line("x 0 0 0 7" + " 0.5" * 16)
    with pytest.raises(ValueError):
        orc.parse_line(" ".join(["1"] * 35))
    text = "\n".join(["# header", "", V1, "bad line", "1 2 3", V2, "  " + V1 + "  \r"]) + "\n"
    el = orc.elites_parse(text)
    assert len(el) == 3 and list(el["id"]) == [1, 2, 1]


def test_model_parse(orc):
    from codec_arena_gb300 import workloads as wl

    w = orc.model_parse(open(wl.SURROGATE_161).read())
    assert len(w) == 161 and w[0] == np.float32(-2.81080210e+01)
    with pytest.raises(ValueError):
        orc.model_parse("152 " + " 0" * 152)
    with pytest.raises(ValueError):
        orc.model_parse("153 " + " 0" * 100)


def _canonical_topk(orc, c, m, el):
    """Brute force: every candidate of every stream, sorted by score desc,
    (stream, index) asc."""
    T = max(1, min(c.threads, c.lambda_))
    per = c.lambda_ // T
    rows = []
    for t in range(T):
        my = c.lambda_ - (T - 1) * per if t == T - 1 else per
        rows.append(orc.stream_dump(c, m, el, t, my))
        rows[-1]["index"] = np.arange(my)
    a = np.concatenate(rows)
    order = np.lexsort((a["index"], a["stream"], -a["score"].astype(np.float64)))
    return a[order][: c.keep]


@pytest.mark.parametrize("lam,T,K,imm,jump", [(5000, 4, 32, 0.01, 0.02), (3000, 7, 100, 0.2, 0.3),
                                              (2000, 1, 10, 0.0, 0.0), (1000, 1000, 5, 1.0, 1.0),
                                              (777, 13, 800, 0.5, 0.5)])
def test_oracle_screen_equals_bruteforce(orc, lam, T, K, imm, jump):
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(16, seed=3)
    m = orc.model_from_compact(wl.seeded_normal_model(seed=4))
    c = orc.cfg(lam, K, 11, threads=T, imm_p=imm, jump_p=jump)
    got, screened = orc.screen(c, m, el)
    want = _canonical_topk(orc, c, m, el)
    assert screened == lam
    assert len(got) == min(K, lam)
    for f in ("score", "stream", "index", "draw", "pa", "pb", "tribe"):
        np.testing.assert_array_equal(got[f], want[f], err_msg=f)
    np.testing.assert_array_equal(got["g"], want["g"])


def test_oracle_walk_matches_dump(orc):
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(8, seed=3)
    m = orc.model_from_compact(wl.seeded_normal_model(seed=4))
    c = orc.cfg(10**6, 4, 9, threads=4)
    d = orc.stream_dump(c, m, el, 2, 500)
    n, nxt = orc.walk(c, 2, 0, int(d["draw"][300]))
    assert n == 300 and nxt == d["draw"][300]
    n, nxt = orc.walk(c, 2, 0, int(d["draw"][300]) + 1)
    assert n == 301 and nxt == d["draw"][301]


def test_oracle_as_shipped_is_empty(orc):
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(8)
    m = orc.model_from_compact(wl.seeded_normal_model())
    got, screened = orc.screen(orc.cfg(1000, 10, 1, flags=orc.FLAG_AS_SHIPPED), m, el)
    assert len(got) == 0 and screened == 1000


def test_oracle_heap_tie_semantics(orc):
    # all-zero surface: every score ties; each stream's heap keeps its first K
    # candidates (`<=` rejects later equals) and the stable sort keeps stream
    # order, so the result is stream 0's first K candidates.
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(8)
    m = orc.model_from_compact(np.zeros(153, np.float32))
    got, _ = orc.screen(orc.cfg(4000, 20, 5, threads=4), m, el)
    assert list(got["stream"]) == [0] * 20
    assert list(got["index"]) == list(range(20))


def test_refit_oracle_pinned_to_reference_refit():
    """oracle/refit.py against brain/evolve.py's own refit_surrogate output
    (400 seeded rows, alpha 50, written with "%.8e")."""
    import json

    import refit

    with open(os.path.join(ROOT, "tests", "golden", "evolve_golden.json")) as f:
        d = json.load(f)
    r = d["refit"]
    assert r["written"]
    for solve in (refit.refit_solve, refit.refit_cholesky):
        w = solve(r["rows_genes"], r["rows_fit"], r["prior"], r["alpha"])
        np.testing.assert_allclose(w, r["weights"], rtol=1e-8, atol=1e-9)
    np.testing.assert_array_equal(refit.features(d["genes"]), np.asarray(d["features"]))
    # fewer than 300 rows: the reference writes nothing (brain/evolve.py:257)
    assert len(r["rows_genes"]) >= 300
