"""The full quadratic surface over all 29 genes (465 compact floats).

No reference code exists for it: docs/RESEARCH_V05C.md:99-102 queues the
quad-block extension ("extend the quad block in v0.6"). Its f32 score is
defined by one FMA order (csx_screen.h); the oracle's orc_score_full follows
that order, and is pinned here to an exact-arithmetic restatement (each fma
rounded once from the exact rational value). The GPU screen and score are
then compared with the oracle bit for bit.
"""
import ctypes
from fractions import Fraction

import numpy as np
import pytest

from conftest import has_gpu

NF = 465


def _round_f32(x: Fraction) -> np.float32:
    """x rounded to the nearest binary32, ties to even (x well inside range)."""
    f = np.float32(float(x))
    cands = [f, np.nextafter(f, np.float32(np.inf)), np.nextafter(f, np.float32(-np.inf))]
    return min(cands, key=lambda c: (abs(Fraction(float(c)) - x), int(np.array(c).view(np.uint32)) & 1))


def _fma(a, b, c) -> np.float32:
    return _round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def _score_exact_order(w, g) -> np.float32:
    w = np.asarray(w, np.float32)
    r = w[0]
    q = 30
    for k in range(29):
        t = w[1 + k]
        for l in range(k + 1):
            t = _fma(w[q + l], g[l], t)
        q += k + 1
        r = _fma(g[k], t, r)
    return r


def _weights(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    return (rng.normal(size=NF) * scale).astype(np.float32)


def test_oracle_score_follows_the_defined_fma_order(orc):
    rng = np.random.default_rng(3)
    for seed in range(3):
        w = _weights(seed)
        m = orc.model_full_from_compact(w)
        for _ in range(6):
            g = rng.random(29).astype(np.float32)
            assert orc.score(m, g).view(np.uint32) == _score_exact_order(w, g).view(np.uint32)


def test_oracle_score_is_the_quadratic_form(orc):
    """The defined order is w0 + sum_k g_k (w_k + sum_{l<=k} Q_kl g_l): the
    FP64 restatement and an independent numpy evaluation agree."""
    rng = np.random.default_rng(4)
    w = _weights(9)
    m = orc.model_full_from_compact(w)
    ii, jj = np.tril_indices(29)
    for _ in range(20):
        g = rng.random(29).astype(np.float32)
        gd = g.astype(np.float64)
        want = float(w[0]) + gd @ w[1:30].astype(np.float64) + (gd[ii] * gd[jj]) @ w[30:].astype(np.float64)
        assert abs(orc.score_f64(m, g) - want) < 1e-9 * (1 + abs(want))
        assert abs(float(orc.score(m, g)) - want) < 1e-3 * (1 + abs(want))


def test_full_model_layout_matches_oracle(csx, orc):
    from codec_arena_gb300 import _lib
    from codec_arena_gb300.screen import ModelFull

    assert ctypes.sizeof(_lib.CsxModelFull) == ctypes.sizeof(orc.OrcModelFull)
    w = _weights(11)
    got, want = ModelFull.from_compact(w), orc.model_full_from_compact(w)
    assert got.w0 == want.w0
    np.testing.assert_array_equal(got.w_lin, np.ctypeslib.as_array(want.w_lin))
    np.testing.assert_array_equal(got.w_quad, np.ctypeslib.as_array(want.w_quad))
    np.testing.assert_array_equal(got.w_quad, w[30:])


@pytest.mark.parametrize("n", [153, 166, 464, 466])
def test_full_model_wrong_size(csx, n):
    from codec_arena_gb300 import CsxError
    from codec_arena_gb300.screen import ModelFull

    with pytest.raises(CsxError) as e:
        ModelFull.from_compact(np.zeros(n, np.float32))
    assert e.value.status == -1


# ---- GPU ------------------------------------------------------------------------

def _check_screen(orc, lam, keep, seed, T, w, el, **kw):
    from codec_arena_gb300 import screen

    cfg = screen.Cfg(lam, keep, seed, threads=T, **kw)
    got, sg = screen.screen(cfg, screen.ModelFull.from_compact(w), el)
    oc = orc.cfg(lam, keep, seed, threads=T, **kw)
    want, sw = orc.screen(oc, orc.model_full_from_compact(w), el, cpu_threads=8)
    assert sg == sw
    assert got.tobytes() == want.tobytes()
    return got


@pytest.mark.gpu
@pytest.mark.parametrize("seed,T,lam,keep,kw", [
    (1, 4, 200_000, 64, {}),
    (2, 1, 50_000, 256, {"imm_p": 0.3, "jump_p": 0.5}),
    (3, 7, 120_000, 32, {"sigma": 0.0}),
    (4, 3, 80_000, 1000, {"sigma": 2.0, "imm_p": 0.0}),
    (5, 64, 30_000, 4096, {"jump_p": 1.0}),
])
def test_gpu_full_screen_equals_oracle(csx, orc, seed, T, lam, keep, kw):
    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import workloads as wl

    _check_screen(orc, lam, keep, seed, T, _weights(100 + seed, 0.3), wl.seeded_elites(32, seed=seed), **kw)


@pytest.mark.gpu
def test_gpu_full_screen_long_segments(csx, orc, monkeypatch):
    """A size whose streams span many walk segments and items."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import workloads as wl

    monkeypatch.setenv("CSX_SEG_CANDS", "700")
    _check_screen(orc, 3_000_000, 128, 17, 4, _weights(21, 0.3), wl.seeded_elites(64))


@pytest.mark.gpu
def test_gpu_full_score_equals_oracle(csx, orc):
    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch
    from codec_arena_gb300 import screen

    w = _weights(5)
    g = torch.rand(5000, 31, device="cuda")
    got = screen.score_genes(screen.ModelFull.from_compact(w), g).cpu().numpy()
    m = orc.model_full_from_compact(w)
    gh = g.cpu().numpy()
    want = np.array([orc.score(m, gh[r, :29]) for r in range(len(gh))], dtype=np.float32)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
def test_gpu_full_screen_refuses_precision_flags(csx):
    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import CsxError, _lib, screen, workloads as wl

    cfg = screen.Cfg(10_000, 16, 1, flags=_lib.FLAG_TC_BF16)
    with pytest.raises(CsxError) as e:
        screen.screen(cfg, screen.ModelFull.from_compact(_weights(1)), wl.seeded_elites(8))
    assert e.value.status == _lib.ERR_BAD_ARGS


@pytest.mark.gpu
@pytest.mark.parametrize("sigma", [1e-31, 2e-40, 3e38, float("inf"), float("nan"), -0.25])
def test_gpu_full_screen_sigma_edge_cases(csx, orc, sigma):
    """Mutation widths outside the fast delta form's range (the exact two-op
    form, NaN genes clamped to 1) on the full surface."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import workloads as wl

    _check_screen(orc, 20_000, 30, 4, 4, _weights(31, 0.3), wl.seeded_elites(64), sigma=sigma)


@pytest.mark.gpu
def test_gpu_cli_takes_a_full_surface_model(csx, tmp_path):
    """`arena screen --model F` with a 465-coefficient file (as
    brain.save_weights writes it) screens on the full surface; the promoted
    file equals the in-process screen's survivors."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import brain, cli, genome, screen, workloads as wl

    w = _weights(44, 0.3).astype(np.float64)
    model_path = tmp_path / "surrogate.txt"
    brain.save_weights(str(model_path), list(w))
    el = wl.seeded_elites(24)
    el_path = tmp_path / "elites.txt"
    el_path.write_text("".join(genome.format_line(r) + "\n" for r in el))
    out, cnt = tmp_path / "promoted.txt", tmp_path / "screens.txt"
    rc = cli.main(["screen", "--model", str(model_path), "--elites", str(el_path), "--out", str(out),
                   "--count-out", str(cnt), "--lambda", "150000", "--keep", "40", "--seed", "77"])
    assert rc == 0 and cnt.read_text() == "150000\n"
    w32 = np.array([np.float32(f"{x:.8e}") for x in w], dtype=np.float32)  # the file's text, as parsed
    cfg = screen.Cfg(150_000, 40, 77)
    want, _ = screen.screen(cfg, screen.ModelFull.from_compact(w32), genome.load_elites_text(el_path.read_text()))
    assert out.read_text() == "".join(screen.format_survivor(r) for r in want)


@pytest.mark.gpu
@pytest.mark.parametrize("lam,T,parts", [(8_000_000, 4, [(0, 1), (1, 3), (3, 4)]), (300_000, 7, [(0, 5), (5, 7)])])
def test_gpu_full_stream_ranges_merge_to_the_generation(csx, lam, T, parts):
    """csx_screen_full_range on a partition of the streams, merged in the
    reference's order, equals the whole full-surface generation bit for bit."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import parallel, screen, workloads as wl

    el = wl.seeded_elites(64)
    m = screen.ModelFull.from_compact(_weights(55, 0.3))
    cfg = screen.Cfg(lam, 96, 13, threads=T)
    whole, n = screen.screen(cfg, m, el)
    pieces = [screen.screen(cfg, m, el, streams=p) for p in parts]
    assert sum(p[1] for p in pieces) == n == lam
    assert parallel.merge_survivors([p[0] for p in pieces], 96).tobytes() == whole.tobytes()
