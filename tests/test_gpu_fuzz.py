"""Seeded random configurations against the oracle: budgets, stream counts,
keep, elite pools, mutation widths, branch probabilities and model layouts
drawn at random; every screen bit-exact (ties at the boundary excepted, as
the reference's per-stream heaps decide them by array position)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")


def _config(i):
    from codec_arena_gb300 import workloads as wl

    rng = np.random.default_rng(1000 + i)
    lam = int(rng.choice([1, 7, 500, 20_000, 300_000, 1_500_000]))
    T = int(rng.choice([1, 2, 3, 4, 9, 64, 1000]))
    keep = int(rng.choice([1, 5, 32, 200, 1024]))
    ne = int(rng.choice([2, 3, 16, 64, 300]))
    n_w = int(rng.choice([153, 159, 161, 164, 165, 166]))
    scale = float(rng.choice([0.1, 1.0, 30.0]))
    w = (rng.normal(0, 1, n_w) * scale).astype(np.float32)
    sigma = float(rng.choice([0.0, 0.01, 0.12, 0.5, 3.0]))
    jump = float(rng.choice([0.0, 0.02, 0.5, 1.0]))
    imm = float(rng.choice([0.0, 0.01, 0.3, 1.0]))
    el = wl.seeded_elites(ne, seed=50 + i)
    return lam, T, keep, w, sigma, jump, imm, el, int(rng.integers(0, 2**63))


@pytest.mark.parametrize("i", range(30))
def test_random_config_matches_oracle(orc, i):
    from codec_arena_gb300 import _lib, screen

    lam, T, keep, w, sigma, jump, imm, el, seed = _config(i)
    flags = _lib.FLAG_EXACT_ALL if i % 5 == 4 else 0
    cfg = screen.Cfg(lam, keep, seed, threads=T, sigma=sigma, jump_p=jump, imm_p=imm, flags=flags)
    got, n = screen.screen(cfg, screen.Model.from_compact(w), el)
    oc = orc.cfg(lam, keep, seed, threads=T, sigma=sigma, jump_p=jump, imm_p=imm)
    want, wn = orc.screen(oc, orc.model_from_compact(w), el, cpu_threads=os.cpu_count() or 4)
    assert n == wn == lam
    # pure crossover (sigma 0, no jumps or immigrants) makes exact f32 ties common;
    # the screen replays the heaps of the streams that hold them
    assert got.tobytes() == want.tobytes()


@pytest.mark.parametrize("b", range(6))
def test_random_batch_matches_single_screens(b):
    """Random batches of the configurations above: every island equals its
    single-island screen bit for bit (the same engine, the same tie order)."""
    from codec_arena_gb300 import _lib, islands, screen

    rng = np.random.default_rng(500 + b)
    picks = rng.choice(30, size=int(rng.integers(2, 9)), replace=False)
    cfgs, models, elites = [], [], []
    for i in picks:
        lam, T, keep, w, sigma, jump, imm, el, seed = _config(int(i))
        cfgs.append(screen.Cfg(lam, keep, seed, threads=T, sigma=sigma, jump_p=jump, imm_p=imm,
                               flags=_lib.FLAG_EXACT_ALL if b == 5 else 0))
        models.append(screen.Model.from_compact(w))
        elites.append(el)
    res = islands.screen_batch(cfgs, models, elites)
    for c, m, e, (surv, n) in zip(cfgs, models, elites, res):
        want, wn = screen.screen(c, m, e)
        assert n == wn
        assert surv.tobytes() == want.tobytes()


@pytest.mark.parametrize("i", range(12))
def test_random_config_full_surface_matches_oracle(orc, i):
    """The same random configurations screened on the full 29-gene surface
    (465 random coefficients) against the oracle's full-surface screen."""
    from codec_arena_gb300 import screen

    lam, T, keep, _, sigma, jump, imm, el, seed = _config(100 + i)
    rng = np.random.default_rng(2000 + i)
    w = (rng.normal(0, 1, 465) * float(rng.choice([0.1, 1.0, 30.0]))).astype(np.float32)
    cfg = screen.Cfg(lam, keep, seed, threads=T, sigma=sigma, jump_p=jump, imm_p=imm)
    got, n = screen.screen(cfg, screen.ModelFull.from_compact(w), el)
    oc = orc.cfg(lam, keep, seed, threads=T, sigma=sigma, jump_p=jump, imm_p=imm)
    want, wn = orc.screen(oc, orc.model_full_from_compact(w), el, cpu_threads=os.cpu_count() or 4)
    assert n == wn == lam
    assert got.tobytes() == want.tobytes()
