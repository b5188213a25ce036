"""The pruning screen on the GPU, through the C ABI.

The default screen skips candidates whose certified bound (from parents and
crossover bits) is below the K-th score; CSX_FLAG_NO_PRUNE scores every
candidate's full synthesis. Both must return the oracle's survivors bit for
bit. Also the reference workload's first configuration exactly as stated
(lambda 1e6, K 32, the seeded 153-coefficient N(0,1) x 0.1 surface from
seed 2, 64 elites from seed 1, seed 7, T = 4) and a 1e8-candidate prefix of
the full generation on that surface.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")


def _run(lam, keep, seed, T, w, el, flags=0, **kw):
    from codec_arena_gb300 import screen

    cfg = screen.Cfg(lam, keep, seed, threads=T, flags=flags, **kw)
    return screen.screen(cfg, screen.Model.from_compact(w), el)


def _orc(orc, lam, keep, seed, T, w, el, **kw):
    c = orc.cfg(lam, keep, seed, threads=T, **kw)
    return orc.screen(c, orc.model_from_compact(w), el, cpu_threads=os.cpu_count() or 4)


def _same(got, want):
    assert len(got) == len(want)
    assert got.tobytes() == want.tobytes()


def _tail_model():
    """A 166-coefficient surface with large linear weights on genes 16..28:
    the bound draws all 29 crossover bits."""
    rng = np.random.default_rng(12)
    w = rng.normal(0, 1, 166).astype(np.float32)
    w[17:30] = rng.normal(0, 20, 13).astype(np.float32)
    return w


def _models():
    from codec_arena_gb300 import workloads as wl

    return {"v3": wl.surrogate_161(), "v1": wl.seeded_normal_model(seed=2), "tail": _tail_model()}


@pytest.mark.parametrize("name", ["v3", "v1", "tail"])
@pytest.mark.parametrize("lam,keep,T", [(2_000_000, 256, 4), (500_000, 1, 7), (300_000, 1000, 1),
                                        (1_000_000, 32, 3000)])
def test_prune_equals_no_prune_and_oracle(orc, name, lam, keep, T):
    """The tensor-core bound (default), the FFMA bound and the unpruned
    screen return the same bytes, and those of the oracle (exact f32 ties
    inside one stream included: the screen replays the stream's heap)."""
    from codec_arena_gb300 import _lib, workloads as wl

    w = _models()[name]
    el = wl.seeded_elites(64)
    a, na = _run(lam, keep, 19, T, w, el)
    f, nf = _run(lam, keep, 19, T, w, el, flags=_lib.FLAG_PRUNE_FFMA)
    b, nb = _run(lam, keep, 19, T, w, el, flags=_lib.FLAG_NO_PRUNE)
    want, nw = _orc(orc, lam, keep, 19, T, w, el)
    assert na == nb == nf == nw == lam
    _same(a, b)
    _same(f, b)
    _same(a, want)


@pytest.mark.parametrize("sigma", [0.0, 0.03, 0.5, 1.5, -0.12, 1e-30])
def test_prune_sigma(orc, sigma):
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(64)
    got, _ = _run(400_000, 64, 3, 4, wl.surrogate_161(), el, sigma=sigma)
    want, _ = _orc(orc, 400_000, 64, 3, 4, wl.surrogate_161(), el, sigma=sigma)
    _same(got, want)


def test_prune_extreme_elites(orc):
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(12)
    el["g"][0, :5] = [-0.0, -3.0, 7.5, np.inf, -np.inf]
    el["g"][1, :3] = [np.nan, 1.0, 0.0]
    el["g"][2, :16] = np.linspace(-0.2, 1.2, 16)
    from codec_arena_gb300 import _lib

    for w in (wl.surrogate_161(), _tail_model()):
        got, _ = _run(500_000, 100, 2, 4, w, el, jump_p=0.3)
        ffma, _ = _run(500_000, 100, 2, 4, w, el, jump_p=0.3, flags=_lib.FLAG_PRUNE_FFMA)
        want, _ = _orc(orc, 500_000, 100, 2, 4, w, el, jump_p=0.3)
        _same(got, want)
        _same(ffma, want)


def test_prune_branch_corners(orc):
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(64)
    for imm, jump in [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0), (0.3, 0.3)]:
        got, _ = _run(300_000, 40, 21, 4, wl.surrogate_161(), el, imm_p=imm, jump_p=jump)
        want, _ = _orc(orc, 300_000, 40, 21, 4, wl.surrogate_161(), el, imm_p=imm, jump_p=jump)
        _same(got, want)


def test_config1_as_stated(orc):
    """The first configuration of the reference workload: 64 elites drawn
    from seed 1, lambda 1e6, the 153-coefficient surface drawn N(0,1) x 0.1
    from seed 2, top 32, seed 7, T = 4, sigma 0.12, jump 0.02, imm 0.01."""
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(64, seed=1)
    w = wl.seeded_normal_model(seed=2, n=153, scale=0.1)
    got, n = _run(1_000_000, 32, 7, 4, w, el)
    want, nw = _orc(orc, 1_000_000, 32, 7, 4, w, el)
    assert n == nw == 1_000_000 and len(got) == 32
    _same(got, want)


def test_config2_seeded_surface_prefix_1e8(orc):
    """The 1e8-candidate prefix of the full generation (T = 4) on the seeded
    N(0, 0.1) 153-coefficient surface, top 256."""
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(64)
    w = wl.seeded_normal_model(seed=2)
    got, n = _run(100_000_000, 256, 7, 4, w, el)
    want, nw = _orc(orc, 100_000_000, 256, 7, 4, w, el)
    assert n == nw
    _same(got, want)


def test_prune_rate_and_full_generation_equal_no_prune():
    """At the bench generation (2.65e9 candidates, T = 4, committed surface,
    top 256) most candidates are skipped, and the survivors of both bounds
    equal the unpruned screen's."""
    from codec_arena_gb300 import _lib, screen, workloads as wl

    el = wl.seeded_elites(64)
    w = wl.surrogate_161()
    a, na = _run(2_650_000_000, 256, 7, 4, w, el, flags=_lib.FLAG_STAGE_TIMES)
    info = screen.last_run_info()
    f, nf = _run(2_650_000_000, 256, 7, 4, w, el, flags=_lib.FLAG_PRUNE_FFMA)
    b, nb = _run(2_650_000_000, 256, 7, 4, w, el, flags=_lib.FLAG_NO_PRUNE)
    assert na == nb == nf == 2_650_000_000
    _same(a, b)
    _same(f, b)
    assert info["exact_evals"] < 0.05 * na, info
