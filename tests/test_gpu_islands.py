"""Batched islands: every island of one batch launch equals the single-island
screen of the same inputs bit for bit (which the single-island tests pin to
the oracle), for any tunables; a few islands are checked against the oracle
directly."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")


def _batch(n, seed, lam_lo, lam_hi, keeps=(32, 128, 256), ne_lo=2, ne_hi=256, sigma=None):
    from codec_arena_gb300 import screen, workloads as wl

    rng = np.random.default_rng(seed)
    isl = wl.seeded_islands(n, seed=seed, lam_lo=lam_lo, lam_hi=lam_hi, ne_lo=ne_lo, ne_hi=ne_hi, keeps=keeps)
    cfgs, models, elites = [], [], []
    for j, d in enumerate(isl):
        sg = float(sigma[j % len(sigma)]) if sigma is not None else float(rng.choice([0.12, 0.05, 0.3]))
        cfgs.append(screen.Cfg(d["lambda"], d["keep"], d["seed"], threads=int(rng.choice([1, 4, 7])), sigma=sg))
        models.append(screen.Model.from_compact(d["weights"]))
        elites.append(d["elites"])
    return cfgs, models, elites


def _same(got, want):
    assert len(got) == len(want)
    np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8))


def _check_against_single(cfgs, models, elites, res):
    from codec_arena_gb300 import screen

    for c, m, e, (surv, n) in zip(cfgs, models, elites, res):
        want, wn = screen.screen(c, m, e)
        assert n == wn == c.lambda_
        _same(surv, want)


def test_batch_matches_single_screens():
    from codec_arena_gb300 import islands

    cfgs, models, elites = _batch(12, 3, 2e3, 3e6)
    res = islands.screen_batch(cfgs, models, elites)
    _check_against_single(cfgs, models, elites, res)
    info = islands.last_batch_info()
    assert info["islands"] == 12 and info["graph_nodes"] > 0 and info["ms_device"] > 0


def test_batch_against_oracle(orc):
    from codec_arena_gb300 import islands

    cfgs, models, elites = _batch(4, 5, 1e4, 4e5)
    res = islands.screen_batch(cfgs, models, elites)
    from codec_arena_gb300 import workloads as wl

    for j, (c, e, (surv, n)) in enumerate(zip(cfgs, elites, res)):
        w = wl.seeded_islands(4, seed=5, lam_lo=1e4, lam_hi=4e5, ne_lo=2, ne_hi=256)[j]["weights"]
        oc = orc.cfg(c.lambda_, c.keep, c.seed, threads=c.threads, sigma=c.sigma, jump_p=c.jump_p, imm_p=c.imm_p)
        want, wn = orc.screen(oc, orc.model_from_compact(w), e, cpu_threads=os.cpu_count() or 4)
        assert n == wn
        _same(surv, want)


@pytest.mark.parametrize("tune", [dict(), dict(ctas_per_sm=1), dict(item_cands=64), dict(seg_cands=700),
                                  dict(item_cands=8192, seg_cands=100000, ctas_per_sm=2)])
def test_tunables_do_not_change_results(tune):
    from codec_arena_gb300 import islands

    cfgs, models, elites = _batch(6, 7, 5e4, 2e6)
    base = islands.screen_batch(cfgs, models, elites)
    got = islands.screen_batch(cfgs, models, elites, tune=islands.Tune(**tune))
    for (a, na), (b, nb) in zip(got, base):
        assert na == nb
        _same(a, b)


def test_pruned_and_unpruned_batch_forms_agree():
    """A batch whose islands all take the tensor-core pruning bound runs one
    pruning screen per island; one island flagged NO_PRUNE sends the whole
    batch through the single unpruned batch kernel. Both equal the single
    screens."""
    import dataclasses

    from codec_arena_gb300 import _lib, islands

    cfgs, models, elites = _batch(7, 21, 2e4, 3e6, keeps=(16, 256, 1000))
    pruned = islands.screen_batch(cfgs, models, elites)
    _check_against_single(cfgs, models, elites, pruned)
    mixed = [dataclasses.replace(c, flags=_lib.FLAG_NO_PRUNE) if j == 3 else c for j, c in enumerate(cfgs)]
    unpruned = islands.screen_batch(mixed, models, elites)
    for (a, na), (b, nb) in zip(pruned, unpruned):
        assert na == nb
        _same(a, b)


def test_pruned_batch_with_a_tail_surface(orc):
    """One island's surface has large linear weights on genes 16..28, so its
    pruning screen draws all 29 crossover bits, beside 16-bit islands and one
    island with 256 elites (two CTAs per SM); every island equals the oracle."""
    from codec_arena_gb300 import screen, islands, workloads as wl

    rng = np.random.default_rng(12)
    tail = rng.normal(0, 1, 166).astype(np.float32)
    tail[17:30] = rng.normal(0, 20, 13).astype(np.float32)
    ws = [tail, wl.surrogate_161(), wl.seeded_normal_model(seed=4)]
    els = [wl.seeded_elites(64, 21), wl.seeded_elites(256, 22), wl.seeded_elites(7, 23)]
    cfgs = [screen.Cfg(900_000, 64, 5, threads=4), screen.Cfg(1_200_000, 128, 6, threads=3),
            screen.Cfg(400_000, 32, 7, threads=5, sigma=0.3)]
    res = islands.screen_batch(cfgs, [screen.Model.from_compact(w) for w in ws], els)
    for c, w, e, (surv, n) in zip(cfgs, ws, els, res):
        oc = orc.cfg(c.lambda_, c.keep, c.seed, threads=c.threads, sigma=c.sigma)
        want, wn = orc.screen(oc, orc.model_from_compact(w), e, cpu_threads=os.cpu_count() or 4)
        assert n == wn == c.lambda_
        _same(surv, want)


def test_edge_islands():
    """Empty budget, budget below keep, two elites, keep 4096, one stream."""
    from codec_arena_gb300 import screen, islands, workloads as wl

    w = wl.seeded_normal_model(seed=9)
    m = screen.Model.from_compact(w)
    cfgs = [screen.Cfg(0, 32, 1), screen.Cfg(17, 32, 2, threads=4), screen.Cfg(50_000, 16, 3, threads=1),
            screen.Cfg(300_000, 4096, 4, threads=5), screen.Cfg(1, 1, 5)]
    elites = [wl.seeded_elites(8, 11), wl.seeded_elites(2, 12), wl.seeded_elites(2, 13), wl.seeded_elites(64, 14),
              wl.seeded_elites(3, 15)]
    res = islands.screen_batch(cfgs, [m] * 5, elites)
    assert res[0][1] == 0 and len(res[0][0]) == 0
    assert len(res[1][0]) == 17 and len(res[4][0]) == 1
    _check_against_single(cfgs[1:], [m] * 4, elites[1:], res[1:])


def test_max_islands_and_graph_reuse():
    from codec_arena_gb300 import islands

    cfgs, models, elites = _batch(64, 8, 1e3, 1e5, keeps=(8, 32))
    res1 = islands.screen_batch(cfgs, models, elites)
    res2 = islands.screen_batch(cfgs, models, elites)  # same shape: the instantiated graph is updated
    for (a, na), (b, nb) in zip(res1, res2):
        assert na == nb
        _same(a, b)
    _check_against_single(cfgs[::9], models[::9], elites[::9], res1[::9])
    small = islands.screen_batch(cfgs[:3], models[:3], elites[:3])  # new shape: a new graph
    for (a, _), (b, _) in zip(small, res1[:3]):
        _same(a, b)


def test_device_api_on_torch_stream():
    import torch

    from codec_arena_gb300 import islands, screen
    from codec_arena_gb300._lib import SURVIVOR_DTYPE

    cfgs, models, elites = _batch(5, 9, 1e4, 1e6)
    flat = np.concatenate(elites)
    d_el = torch.from_numpy(flat.view(np.uint8).copy()).cuda()
    keeps = [c.keep for c in cfgs]
    d_out = torch.zeros(sum(keeps) * SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4 * len(cfgs), dtype=torch.int64, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        islands.screen_batch_device(cfgs, models, d_el, [len(e) for e in elites], d_out, d_res)
    s.synchronize()
    res = d_res.cpu().numpy().reshape(-1, 4)
    out = d_out.cpu().numpy().view(SURVIVOR_DTYPE)
    off = 0
    for i, (c, m, e) in enumerate(zip(cfgs, models, elites)):
        assert res[i, 2] == 0 and res[i, 1] == c.lambda_
        want, _ = screen.screen(c, m, e)
        _same(out[off: off + int(res[i, 0])], want)
        off += keeps[i]


def test_batch_errors():
    from codec_arena_gb300 import _lib, islands, screen, workloads as wl

    m = screen.Model.from_compact(wl.seeded_normal_model())
    with pytest.raises(_lib.CsxError) as e:
        islands.screen_batch([screen.Cfg(10, 2, 1)], [m], [wl.seeded_elites(1)])
    assert e.value.status == _lib.ERR_NEED_TWO_ELITES
    with pytest.raises(_lib.CsxError) as e:
        islands.screen_batch([screen.Cfg(10, 2, 1)] * 65, [m] * 65, [wl.seeded_elites(4)] * 65)
    assert e.value.status == _lib.ERR_LIMIT
    with pytest.raises(_lib.CsxError) as e:
        islands.screen_batch([screen.Cfg(10, 0, 1)], [m], [wl.seeded_elites(4)])
    assert e.value.status == _lib.ERR_BAD_ARGS


def test_autotune_on_gpu(tmp_path, monkeypatch):
    from codec_arena_gb300 import autotune, islands

    monkeypatch.setenv("CSX_TUNE_CACHE", str(tmp_path / "tune.json"))
    cfgs, models, elites = _batch(4, 10, 1e5, 1e6)
    best, table = autotune.autotune(cfgs, models, elites, candidates=autotune.CANDIDATES[:3], reps=1)
    assert best in autotune.CANDIDATES[:3] and len(table) == 3
    again, _ = autotune.autotune(cfgs, models, elites, candidates=autotune.CANDIDATES[:3], reps=1)
    assert again == best  # from the cache
    res = islands.screen_batch(cfgs, models, elites, tune=best)
    _check_against_single(cfgs, models, elites, res)
