"""Precision form: tensor-core (tcgen05) scoring in BF16 / FP16 against a
numpy emulation of the same rounded inputs (tight: only FP32 accumulation
differs) and against the FP64 score (the error the form trades)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")


def _round(x, form):
    import torch

    t = torch.from_numpy(np.asarray(x, dtype=np.float32))
    return t.to(torch.bfloat16 if form == "bf16" else torch.float16).to(torch.float64).numpy()


def _emulate(model, g, form):
    """FP64 evaluation of the precision form on the same rounded operands."""
    g = g.astype(np.float64)
    w0, lin, q = float(model.w0), model.w_lin.astype(np.float64), model.w_quad.astype(np.float64).reshape(16, 16)
    L = np.tril(q)
    s = 16 * w0 + g @ lin
    if form == "bf16":
        x = _round(g[:, :16], "bf16")
        y = x @ _round(L, "bf16").T
        return s + np.sum(g[:, :16] * y, axis=1), np.abs(16 * w0) + np.abs(g) @ np.abs(lin) + \
            np.sum(np.abs(g[:, :16]) * (np.abs(x) @ np.abs(L).T), axis=1)
    xp = 2 * g[:, :16] - 1
    u = (L.sum(axis=1) + L.sum(axis=0)) / 4
    v = L.sum() / 4
    c = 16 * w0 + v - u.sum()
    lin2 = lin.copy()
    lin2[:16] += 2 * u
    cf = np.float32(c).astype(np.float64)
    lf = lin2.astype(np.float32).astype(np.float64)
    y = _round(xp, "fp16") @ _round(L / 4, "fp16").T
    A = np.abs(cf) + np.abs(g) @ np.abs(lf) + np.sum(np.abs(xp) * (np.abs(xp) @ np.abs(L / 4).T), axis=1)
    return cf + g @ lf + np.sum(xp * y, axis=1), A


def _fp64(model, g):
    g = g.astype(np.float64)
    L = np.tril(model.w_quad.astype(np.float64).reshape(16, 16))
    return 16 * float(model.w0) + g @ model.w_lin.astype(np.float64) + np.einsum("ni,ij,nj->n", g[:, :16], L, g[:, :16])


@pytest.mark.parametrize("form", ["bf16", "fp16"])
@pytest.mark.parametrize("which", ["v3", "normal"])
def test_tc_score_matches_emulation_and_bounds(form, which):
    import torch

    from codec_arena_gb300 import precision, screen, workloads as wl

    w = wl.surrogate_161() if which == "v3" else wl.seeded_normal_model(seed=2)
    m = screen.Model.from_compact(w)
    rng = np.random.default_rng(3)
    n = 100_003
    g = rng.random((n, 29), dtype=np.float32)
    got = precision.tc_score(m, torch.from_numpy(g).cuda(), form).cpu().numpy().astype(np.float64)
    emu, A = _emulate(m, g, form)
    assert np.all(np.abs(got - emu) <= 2e-6 * A), np.max(np.abs(got - emu) / A)
    exact = _fp64(m, g)
    Ax = np.abs(16 * float(m.w0)) + np.abs(g.astype(np.float64)) @ np.abs(m.w_lin.astype(np.float64)) + \
        np.einsum("ni,ij,nj->n", np.abs(g[:, :16].astype(np.float64)), np.abs(np.tril(m.w_quad.reshape(16, 16))),
                  np.abs(g[:, :16].astype(np.float64)))
    rel = np.abs(got - exact) / Ax
    bound = 3 * 2.0 ** -8 if form == "bf16" else 3 * 2.0 ** -11
    assert rel.max() <= bound, (rel.max(), bound)
    # a padded row stride and a ragged tail
    g2 = np.zeros((1000, 32), np.float32)
    g2[:, :29] = g[:1000]
    got2 = precision.tc_score(m, torch.from_numpy(g2).cuda(), form).cpu().numpy()
    np.testing.assert_array_equal(got2, got[:1000].astype(np.float32))


def _truth(orc, w, el, lam, K, seed, T, sigma=0.12):
    """Every candidate from the oracle, scored in FP64; the FP64 top-K by
    (score desc, stream, index)."""
    c = orc.cfg(lam, K, seed, threads=T, sigma=sigma)
    m = orc.model_from_compact(w)
    per = lam // T
    cands = np.concatenate([orc.stream_dump(c, m, el, t, per if t < T - 1 else lam - (T - 1) * per)
                            for t in range(T)])
    from codec_arena_gb300 import screen

    s64 = _fp64(screen.Model.from_compact(w), cands["g"])
    order = np.lexsort((cands["index"], cands["stream"], -s64))
    return cands, s64, order


@pytest.mark.parametrize("form,which", [("bf16", "v3"), ("fp16", "v3"), ("bf16", "normal"), ("fp16", "normal")])
def test_tc_screen_is_fp64_top_k(orc, form, which):
    """The precision screen returns the FP64 top-K: its band (max of 1e-3
    relative and the form's certified error bound) never drops a candidate of
    the FP64 top-K. Genes and lineage are bit-exact; scores are the FP64 score
    rounded to f32."""
    from codec_arena_gb300 import _lib, screen, workloads as wl

    w = wl.surrogate_161() if which == "v3" else wl.seeded_normal_model(seed=2)
    el = wl.seeded_elites(64)
    lam, K, T, seed = 600_000, 256, 4, 7
    flag = _lib.FLAG_TC_BF16 if form == "bf16" else _lib.FLAG_TC_FP16
    got, n = screen.screen(screen.Cfg(lam, K, seed, threads=T, flags=flag), screen.Model.from_compact(w), el)
    assert n == lam and len(got) == K
    cands, s64, order = _truth(orc, w, el, lam, K, seed, T)
    pos = {(int(cands["stream"][i]), int(cands["index"][i])): i for i in order[: 4 * K]}
    for r in got:
        i = pos[(int(r["stream"]), int(r["index"]))]
        assert r["g"].tobytes() == cands["g"][i].tobytes()
        assert (r["pa"], r["pb"], r["tribe"], r["draw"]) == (cands["pa"][i], cands["pb"][i], cands["tribe"][i],
                                                               cands["draw"][i])
        assert abs(float(r["score"]) - s64[i]) <= abs(s64[i]) * 2 ** -23
    want = {(int(cands["stream"][i]), int(cands["index"][i])) for i in order[:K]}
    have = {(int(r["stream"]), int(r["index"])) for r in got}
    # ties at f32 resolution of the K-th FP64 score may swap members; otherwise the sets agree
    kth = np.float32(s64[order[K - 1]])
    diff = (want ^ have)
    assert all(np.float32(s64[pos[k]] if k in pos else -np.inf) == kth for k in diff), len(diff)
    scores = got["score"]
    assert np.all(scores[:-1] >= scores[1:])


def test_tc_screen_deterministic_and_counts():
    from codec_arena_gb300 import _lib, screen, workloads as wl

    w = wl.surrogate_161()
    el = wl.seeded_elites(64)
    cfg = screen.Cfg(3_000_000, 128, 11, threads=4, flags=_lib.FLAG_TC_FP16)
    a, na = screen.screen(cfg, screen.Model.from_compact(w), el)
    b, nb = screen.screen(cfg, screen.Model.from_compact(w), el)
    assert na == nb == 3_000_000
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("form", ["bf16", "fp16"])
def test_pruned_precision_form_equals_unpruned(form):
    """The precision form prunes with its tile format's bound and ranks queued
    candidates by their FP64 score; the unpruned precision kernel
    (CSX_FLAG_NO_PRUNE) scores every candidate on the tensor cores with an FP64
    band. Both certify the FP64 top-K, so their survivors are the same bytes,
    on the committed surface, a surface with linear weights past gene 15 and
    elites with genes outside [0, 1]."""
    from codec_arena_gb300 import _lib, screen, workloads as wl

    flag = _lib.FLAG_TC_BF16 if form == "bf16" else _lib.FLAG_TC_FP16
    rng = np.random.default_rng(12)
    tail = rng.normal(0, 1, 166).astype(np.float32)
    tail[17:30] = rng.normal(0, 20, 13).astype(np.float32)
    odd = wl.seeded_elites(12)
    odd["g"][0, :5] = [-0.0, -3.0, 7.5, np.inf, -np.inf]
    odd["g"][1, :3] = [np.nan, 1.0, 0.0]
    for w, el, lam, K, T in ((wl.surrogate_161(), wl.seeded_elites(64), 3_000_000, 256, 4),
                             (tail, wl.seeded_elites(64), 1_000_000, 64, 7),
                             (wl.surrogate_161(), odd, 1_000_000, 100, 3)):
        m = screen.Model.from_compact(w)
        a, na = screen.screen(screen.Cfg(lam, K, 5, threads=T, flags=flag), m, el)
        b, nb = screen.screen(screen.Cfg(lam, K, 5, threads=T, flags=flag | _lib.FLAG_NO_PRUNE), m, el)
        assert na == nb == lam and len(a) == K
        assert a.tobytes() == b.tobytes()
