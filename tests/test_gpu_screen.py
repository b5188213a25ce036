"""GPU screen vs the CPU oracle, through the C ABI (bit-exact).

Survivors are compared field by field: score and gene bit patterns, lineage,
stream, stream-local index and draw position. Sizes are ones the oracle
finishes in seconds; the full-size generation is checked through properties
(count, order, per-survivor regeneration by the oracle).
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


def _models():
    from codec_arena_gb300 import workloads as wl

    rng = np.random.default_rng(66)
    return {
        "v1_normal": wl.seeded_normal_model(seed=2),
        "v3_committed": wl.surrogate_161(),
        "v6_random": rng.normal(0, 3, 166).astype(np.float32),
    }


def _gpu(lam, keep, seed, T, w, el, sigma=0.12, jump=0.02, imm=0.01, flags=0):
    from codec_arena_gb300 import screen

    cfg = screen.Cfg(lam, keep, seed, threads=T, sigma=sigma, jump_p=jump, imm_p=imm, flags=flags)
    return screen.screen(cfg, screen.Model.from_compact(w), el)


def _orc(orc, lam, keep, seed, T, w, el, sigma=0.12, jump=0.02, imm=0.01, flags=0):
    c = orc.cfg(lam, keep, seed, threads=T, sigma=sigma, jump_p=jump, imm_p=imm, flags=flags)
    return orc.screen(c, orc.model_from_compact(w), el, cpu_threads=os.cpu_count() or 4)


def assert_same(got, want):
    assert len(got) == len(want), (len(got), len(want))
    np.testing.assert_array_equal(got["score"].view(np.uint32), want["score"].view(np.uint32))
    for f in ("stream", "index", "draw", "pa", "pb", "tribe"):
        np.testing.assert_array_equal(got[f], want[f], err_msg=f)
    np.testing.assert_array_equal(got["g"].view(np.uint32), want["g"].view(np.uint32))


def check(orc, *args, **kw):
    got, sg = _gpu(*args, **kw)
    want, sw = _orc(orc, *args, **kw)
    assert sg == sw
    assert_same(got, want)
    return got


@pytest.fixture
def env(monkeypatch):
    return monkeypatch


def test_basic_t4(orc):
    from codec_arena_gb300 import workloads as wl

    check(orc, 100_000, 32, 7, 4, wl.seeded_normal_model(), wl.seeded_elites(64))


@pytest.mark.parametrize("name", ["v1_normal", "v3_committed", "v6_random"])
def test_models(orc, name):
    from codec_arena_gb300 import workloads as wl

    check(orc, 60_000, 192, 3, 4, _models()[name], wl.seeded_elites(64))


@pytest.mark.parametrize("T", [1, 2, 3, 7, 64, 999, 5000, 20000])
def test_stream_counts(orc, T):
    from codec_arena_gb300 import workloads as wl

    check(orc, 20_000, 50, 11, T, wl.surrogate_161(), wl.seeded_elites(32))


def test_one_candidate_per_stream(orc):
    from codec_arena_gb300 import workloads as wl

    check(orc, 3000, 40, 5, 3000, wl.surrogate_161(), wl.seeded_elites(16))
    check(orc, 3000, 40, 5, 10**9, wl.surrogate_161(), wl.seeded_elites(16))


@pytest.mark.parametrize("seg,item", [(500, 64), (37, 64), (3, 64), (1, 64), (2000, 4096)])
def test_segment_linking(orc, env, seg, item):
    """Short segments force the walk's meeting-point logic, including chains
    that meet only several segments later."""
    from codec_arena_gb300 import workloads as wl

    env.setenv("CSX_SEG_CANDS", str(seg))
    env.setenv("CSX_ITEM_CANDS", str(item))
    check(orc, 40_000, 64, 9, 4, wl.surrogate_161(), wl.seeded_elites(64))
    check(orc, 7_001, 20, 1, 3, wl.seeded_normal_model(), wl.seeded_elites(5), imm=0.3, jump=0.4)


@pytest.mark.parametrize("seg", [1, 3, 37, 300])
def test_every_candidate_once(orc, env, seg):
    """keep = lambda: every candidate survives, so the survivor list is the
    whole generation. Segments of a few candidates make nearly every
    boundary meet past the next segment's walk checkpoints, and the items of
    64 candidates split every segment's range: each candidate must appear
    once, with its stream, index, draw, parents and genes. 4096 scores near
    -380 hold exact f32 ties, whose order inside one stream the reference's
    heap decides: the screen replays those heaps, so the order is exact."""
    from codec_arena_gb300 import workloads as wl

    env.setenv("CSX_SEG_CANDS", str(seg))
    env.setenv("CSX_ITEM_CANDS", "64")
    got = check(orc, 4096, 4096, 31, 2, wl.surrogate_161(), wl.seeded_elites(16), imm=0.2, jump=0.3)
    assert len(got) == 4096
    keys = {(int(r["stream"]), int(r["index"])) for r in got}
    assert keys == {(t, i) for t in range(2) for i in range(2048)}


@pytest.mark.parametrize("imm,jump", [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0), (0.0, 0.02),
                                      (0.5, 0.5), (0.01, 0.0), (1e-7, 0.02), (float("nan"), 2.0)])
def test_branch_probabilities(orc, env, imm, jump):
    from codec_arena_gb300 import workloads as wl

    env.setenv("CSX_SEG_CANDS", "300")
    check(orc, 30_000, 40, 21, 4, wl.surrogate_161(), wl.seeded_elites(64), imm=imm, jump=jump)


@pytest.mark.parametrize("sigma", [0.0, 0.5, 1e-30, 1e-31, 2e-40, 2.0, 3e38, float("inf"), float("nan"), -0.25])
def test_sigma(orc, sigma):
    from codec_arena_gb300 import workloads as wl

    check(orc, 20_000, 30, 4, 4, wl.surrogate_161(), wl.seeded_elites(64), sigma=sigma)


@pytest.mark.parametrize("keep", [1, 2, 31, 192, 1000, 4096])
def test_keep(orc, keep):
    from codec_arena_gb300 import workloads as wl

    check(orc, 50_000, keep, 8, 4, wl.seeded_normal_model(), wl.seeded_elites(64))


@pytest.mark.parametrize("ne", [2, 3, 17, 256, 1536])
def test_elite_counts(orc, ne):
    from codec_arena_gb300 import workloads as wl

    check(orc, 30_000, 64, 12, 4, wl.surrogate_161(), wl.seeded_elites(ne, seed=ne))


def test_small_lambda(orc):
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(8)
    w = wl.surrogate_161()
    got = check(orc, 5, 100, 1, 4, w, el)      # fewer candidates than keep
    assert len(got) == 5
    got = check(orc, 1, 3, 1, 4, w, el)
    assert len(got) == 1
    got, s = _gpu(0, 10, 1, 4, w, el)
    assert len(got) == 0 and s == 0


def test_all_ties(orc):
    """Zero surface: every score is 0. Ties go to (stream, index); the
    reference's heaps keep each stream's first K and its stable sort keeps
    stream order, which is the same list."""
    from codec_arena_gb300 import workloads as wl

    got = check(orc, 40_000, 100, 3, 4, np.zeros(153, np.float32), wl.seeded_elites(8))
    assert list(got["index"]) == list(range(100))


def test_elites_with_extreme_genes(orc):
    from codec_arena_gb300 import genome, workloads as wl

    el = wl.seeded_elites(12)
    el["g"][0, :5] = [-0.0, -3.0, 7.5, np.inf, -np.inf]
    el["g"][1, :3] = [np.nan, 1.0, 0.0]
    check(orc, 20_000, 50, 2, 4, wl.surrogate_161(), el)


def test_as_shipped(orc):
    from codec_arena_gb300 import _lib, workloads as wl

    got, s = _gpu(10_000, 10, 1, 4, wl.surrogate_161(), wl.seeded_elites(8), flags=_lib.FLAG_AS_SHIPPED)
    assert len(got) == 0 and s == 10_000


def test_repeatable_and_buffer_regrowth(orc):
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(64)
    w = wl.surrogate_161()
    a, _ = _gpu(200_000, 256, 5, 4, w, el)
    _gpu(1000, 4000, 5, 2, w, el)
    _gpu(100, 3, 5, 100, w, wl.seeded_elites(1500))
    b, _ = _gpu(200_000, 256, 5, 4, w, el)
    assert a.tobytes() == b.tobytes()


def test_prefix_1e8_t4(orc):
    """The 1e8-candidate prefix of the full generation, T = 4 (the reference
    CI's stream count), committed surrogate, 64 seeded elites, top 256."""
    from codec_arena_gb300 import workloads as wl

    check(orc, 100_000_000, 256, 7, 4, wl.surrogate_161(), wl.seeded_elites(64))


def test_full_generation_properties(orc):
    """2.65e9 candidates, T = 2^20 streams (short streams, so the oracle can
    re-walk each survivor's stream): count, order, and every survivor
    regenerated by the oracle from (stream, draw) with its index re-walked."""
    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(64)
    w = wl.surrogate_161()
    lam, T = 2_650_000_000, 1 << 20
    got, screened = _gpu(lam, 256, 7, T, w, el)
    assert screened == lam and len(got) == 256
    s = got["score"].astype(np.float64)
    assert np.all(s[:-1] >= s[1:])
    c = orc.cfg(lam, 256, 7, threads=T)
    m = orc.model_from_compact(w)
    for r in got:
        o, _ = orc.candidate(c, m, el, int(r["stream"]), int(r["draw"]))
        assert o["score"].view(np.uint32) == r["score"].view(np.uint32)
        assert o["g"].tobytes() == r["g"].tobytes()
        assert (o["pa"], o["pb"], o["tribe"]) == (r["pa"], r["pb"], r["tribe"])
        n, nxt = orc.walk(c, int(r["stream"]), 0, int(r["draw"]))
        assert n == r["index"] and nxt == r["draw"]


def test_cli_end_to_end(orc, tmp_path):
    from codec_arena_gb300 import cli, genome, screen, workloads as wl

    seed_pop = os.path.join(wl.GOLDEN_DIR, "pop_seed_96.txt")
    for extra, flags, fix in (([], 0, False), (["--compat-29"], 2, False), (["--parse-v6-fix"], 0, True)):
        out, cnt = tmp_path / "p.txt", tmp_path / "c.txt"
        rc = cli.main(["screen", "--model", wl.SURROGATE_161, "--elites", seed_pop, "--out", str(out),
                       "--count-out", str(cnt), "--lambda", "300000", "--keep", "192", "--seed", "7",
                       "--threads", "4", *extra])
        assert rc == 0
        assert cnt.read_text() == "300000\n"
        el = genome.load_elites(seed_pop, v6_fix=fix)
        want, _ = _orc(orc, 300_000, 192, 7, 4, wl.surrogate_161(), el)
        lines = out.read_text().splitlines(keepends=True)
        assert len(lines) == 192
        assert lines == [screen.format_survivor(r, flags) for r in want]


def test_screen_device_torch_stream(orc):
    import torch

    from codec_arena_gb300 import _lib, screen, workloads as wl

    el = wl.seeded_elites(64)
    w = wl.surrogate_161()
    cfg = screen.Cfg(150_000, 100, 4, threads=4)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    d_out = torch.zeros(100 * _lib.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        screen.screen_device(cfg, screen.Model.from_compact(w), d_el, d_out, d_res)
    s.synchronize()
    res = d_res.cpu().numpy()
    assert res[2] == 0 and res[1] == 150_000
    got = screen.survivors_from_bytes(d_out.cpu().numpy(), int(res[0]))
    want, _ = _orc(orc, 150_000, 100, 4, 4, w, el)
    assert_same(got, want)


@pytest.mark.parametrize("flags", [0, 8])
def test_filter_and_exact_modes(orc, flags):
    """Default mode scores with a certified FFMA filter and re-evaluates the
    reference order only near the threshold; CSX_FLAG_EXACT_ALL (8) evaluates
    the reference order for every candidate. Both must equal the oracle."""
    from codec_arena_gb300 import workloads as wl

    check(orc, 300_000, 256, 17, 4, wl.surrogate_161(), wl.seeded_elites(64), flags=flags)


def test_filter_wide_dynamic_range(orc):
    """Coefficients spanning 1e-6..1e6 with cancelling signs: large rounding
    differences between the two evaluation orders."""
    from codec_arena_gb300 import workloads as wl

    rng = np.random.default_rng(3)
    w = (rng.choice([-1.0, 1.0], 166) * 10.0 ** rng.uniform(-6, 6, 166)).astype(np.float32)
    w[0] = 1e5
    for keep in (1, 64):
        check(orc, 200_000, keep, 5, 4, w, wl.seeded_elites(64))


def test_filter_near_ties(orc):
    """A surface with few distinct values (integer weights, genes snapped by
    clamping) makes many scores tie or nearly tie at the threshold."""
    from codec_arena_gb300 import workloads as wl

    w = np.zeros(153, np.float32)
    w[1:17] = 1.0
    el = wl.seeded_elites(8)
    el["g"][:] = np.where(el["g"] > 0.5, 2.0, -1.0)
    got = check(orc, 100_000, 200, 3, 4, w, el, sigma=0.1, imm=0.0, jump=0.0)
    assert len(np.unique(got["score"])) < len(got)  # the case really has ties


def test_late_meetings_block_assembly(orc, env):
    """Segments of 2000 candidates are shorter than a typical meeting of two
    chains (~3.3k candidates per chain), so many segments are late: their
    incoming meeting lies past their outgoing one. The block assembly repairs
    those runs locally; the survivors must still equal the oracle's."""
    from codec_arena_gb300 import workloads as wl

    env.setenv("CSX_SEG_CANDS", "2000")
    check(orc, 20_000_000, 128, 23, 4, wl.surrogate_161(), wl.seeded_elites(64))
    env.setenv("CSX_SEG_CANDS", "700")
    check(orc, 6_000_000, 64, 5, 3, wl.seeded_normal_model(), wl.seeded_elites(20), imm=0.05, jump=0.1)


@pytest.mark.parametrize("lam,T,parts", [(30_000_000, 4, [(0, 1), (1, 2), (2, 3), (3, 4)]),
                                         (30_000_000, 4, [(0, 3), (3, 4)]),
                                         (5_000_003, 7, [(0, 2), (2, 7)]),
                                         (90_000, 5, [(0, 4), (4, 5)]),
                                         (1_000, 3, [(1, 3), (0, 1)])])
def test_stream_ranges_merge_to_the_generation(lam, T, parts):
    """csx_screen_range on a partition of the streams, merged in the
    reference's order, equals the whole generation bit for bit."""
    from codec_arena_gb300 import parallel, screen, workloads as wl

    el = wl.seeded_elites(64)
    m = screen.Model.from_compact(wl.surrogate_161())
    cfg = screen.Cfg(lam, 128, 31, threads=T)
    full, n = screen.screen(cfg, m, el)
    pieces = [screen.screen(cfg, m, el, streams=p) for p in parts]
    assert sum(p[1] for p in pieces) == n == lam
    for (surv, _), (a, b) in zip(pieces, parts):
        assert np.all((surv["stream"] >= a) & (surv["stream"] < b))
    assert parallel.merge_survivors([p[0] for p in pieces], 128).tobytes() == full.tobytes()


@pytest.mark.parametrize("lam,T,W", [(30_000_000, 4, 2), (30_000_000, 4, 7), (5_000_003, 2, 3), (1_000, 3, 5),
                                     (20, 4, 9)])
def test_item_shards_merge_to_the_generation(lam, T, W):
    """csx_screen_items: W shares of the generation's work items (W may exceed
    the stream count and the item count), merged in the reference's order,
    equal the whole generation bit for bit; the shares' screened counts sum
    to lambda."""
    from codec_arena_gb300 import parallel, screen, workloads as wl

    el = wl.seeded_elites(64)
    m = screen.Model.from_compact(wl.surrogate_161())
    cfg = screen.Cfg(lam, 128, 31, threads=T)
    full, n = screen.screen(cfg, m, el)
    pieces = [screen.screen(cfg, m, el, items=parallel.item_shard(r, W)) for r in range(W)]
    assert sum(p[1] for p in pieces) == n == lam
    assert parallel.merge_survivors([p[0] for p in pieces], 128).tobytes() == full.tobytes()


def test_stream_range_errors():
    from codec_arena_gb300 import _lib, screen, workloads as wl

    m = screen.Model.from_compact(wl.surrogate_161())
    el = wl.seeded_elites(8)
    for rg in [(3, 1), (0, 5)]:
        with pytest.raises(_lib.CsxError) as e:
            screen.screen(screen.Cfg(1000, 8, 1, threads=4), m, el, streams=rg)
        assert e.value.status == _lib.ERR_BAD_ARGS
    # an empty range (a rank with no stream of its own) screens nothing
    surv, n = screen.screen(screen.Cfg(1000, 8, 1, threads=4), m, el, streams=(2, 2))
    assert len(surv) == 0 and n == 0
    for sh in [(0, 0), (3, 3)]:
        with pytest.raises(_lib.CsxError) as e:
            screen.screen(screen.Cfg(1000, 8, 1, threads=4), m, el, items=sh)
        assert e.value.status == _lib.ERR_BAD_ARGS


@pytest.mark.slow
def test_makefile_screen_target(orc, tmp_path):
    """The reference's `make screen` (Makefile:21-22): arena screen --model
    state/surrogate.txt --elites pop/seed.txt --lambda 100000000 --keep 192
    --seed 7 --threads 4, through this repository's CLI, equals the oracle's
    promoted lines and count file."""
    from codec_arena_gb300 import cli, genome, screen, workloads as wl

    seed_pop = os.path.join(wl.GOLDEN_DIR, "pop_seed_96.txt")
    out, cnt = tmp_path / "promoted.txt", tmp_path / "screens.txt"
    rc = cli.main(["screen", "--model", wl.SURROGATE_161, "--elites", seed_pop, "--out", str(out),
                   "--count-out", str(cnt), "--lambda", "100000000", "--keep", "192", "--seed", "7",
                   "--threads", "4"])
    assert rc == 0
    assert cnt.read_text() == "100000000\n"
    el = genome.load_elites(seed_pop)
    want, n = _orc(orc, 100_000_000, 192, 7, 4, wl.surrogate_161(), el)
    assert n == 100_000_000
    assert out.read_text().splitlines(keepends=True) == [screen.format_survivor(r) for r in want]


def test_score_genes_in_reference_order(orc):
    """csx_score equals the oracle's Model.score bit for bit, on random genes
    and on genes with exact 0s and 1s."""
    import torch

    from codec_arena_gb300 import screen

    rng = np.random.default_rng(71)
    for w in _models().values():
        m = screen.Model.from_compact(w)
        om = orc.model_from_compact(w)
        g = rng.random((3000, 29), dtype=np.float32)
        g[::7] = np.round(g[::7])
        got = screen.score_genes(m, torch.from_numpy(g).cuda()).cpu().numpy()
        want = np.array([orc.score(om, row) for row in g], dtype=np.float32)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_link_failure_voids_the_call_and_skips_the_screen(orc, env):
    """A link that runs out of steps (CSX_LINK_CAP lowered to 1 on segments of
    3 candidates) sets the link error bit; assembly stops at the failed
    segment, the scan emits no item, the screen screens nothing, and the call
    returns ERR_DEVICE_STATE. The context stays usable: the next call, at the
    default cap, equals the oracle. No GPU fault is involved."""
    import torch

    from codec_arena_gb300 import _lib, screen, workloads as wl

    el = wl.seeded_elites(64)
    w = wl.surrogate_161()
    env.setenv("CSX_SEG_CANDS", "3")
    env.setenv("CSX_LINK_CAP", "1")
    with pytest.raises(_lib.CsxError) as e:
        _gpu(100_000, 32, 5, 4, w, el)
    assert e.value.status == _lib.ERR_DEVICE_STATE
    cfg = screen.Cfg(100_000, 32, 5, threads=4)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    d_out = torch.zeros(32 * _lib.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    screen.screen_device(cfg, screen.Model.from_compact(w), d_el, d_out, d_res)
    torch.cuda.synchronize()
    res = d_res.cpu().numpy()
    assert res[2] & 1 and res[1] == 0 and res[3] == 0  # link bit; nothing screened, no item
    env.delenv("CSX_LINK_CAP")
    check(orc, 100_000, 32, 5, 4, w, el)


@pytest.mark.parametrize("T,keep,lam", [(1, 1000, 300_000), (3, 500, 200_000), (4, 64, 2_000_000)])
def test_exact_ties_follow_the_reference_heap(orc, T, keep, lam):
    """Integer-valued surfaces make many candidates of one stream tie exactly,
    inside the kept list and at the K-th score. The reference ranks them by
    its per-stream heap (array order, and which tied candidates the heap kept)
    and the screen replays those heaps: the survivors equal the oracle's
    byte for byte, for the whole generation and for stream ranges merged."""
    from codec_arena_gb300 import parallel, screen, workloads as wl

    w = np.zeros(153, np.float32)
    w[1:17] = np.arange(16) % 3
    w[17:30] = np.arange(13) % 2
    el = wl.seeded_elites(8, seed=4)
    el["g"][:] = np.where(el["g"] > 0.5, 2.0, -1.0)  # genes clamp to 0 or 1: integer scores
    kw = dict(sigma=0.1, imm=0.0, jump=0.0)
    got = check(orc, lam, keep, 9, T, w, el, **kw)
    assert len(np.unique(got["score"])) < len(got) // 4  # the case is tie-heavy
    if T > 1:
        cfg = screen.Cfg(lam, keep, 9, threads=T, sigma=0.1, imm_p=0.0, jump_p=0.0)
        m = screen.Model.from_compact(w)
        parts = [screen.screen(cfg, m, el, streams=rg)[0] for rg in ((0, 1), (1, T))]
        assert parallel.merge_survivors(parts, keep).tobytes() == got.tobytes()


def test_small_generations_take_the_unpruned_form(orc, env):
    """Without the tests' floor the library screens a small generation with
    the unpruned filter kernel (two CTAs per SM) and a large one with the
    pruning screen (three), which a floor of 0 selects at every size; the
    small one equals the oracle."""
    from codec_arena_gb300 import screen, workloads as wl

    w = wl.seeded_normal_model(seed=2)
    el = wl.seeded_elites(64, seed=1)
    env.setenv("CSX_PRUNE_MIN_CANDS", "0")  # the tests' floor: prune at every size
    screen.screen(screen.Cfg(1_000_000, 32, 7, threads=4), screen.Model.from_compact(w), el)
    forced = screen.last_run_info()
    env.delenv("CSX_PRUNE_MIN_CANDS", raising=False)
    got, n = screen.screen(screen.Cfg(1_000_000, 32, 7, threads=4), screen.Model.from_compact(w), el)
    small = screen.last_run_info()
    want, wn = orc.screen(orc.cfg(1_000_000, 32, 7, threads=4), orc.model_from_compact(w), el,
                          cpu_threads=os.cpu_count() or 4)
    assert n == wn and got.tobytes() == want.tobytes()
    screen.screen(screen.Cfg(100_000_000, 32, 7, threads=4), screen.Model.from_compact(w), el)
    large = screen.last_run_info()
    assert small["screen_ctas"] < large["screen_ctas"] == forced["screen_ctas"], (small, large, forced)
