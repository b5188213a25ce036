"""The in-process screen step and the file formats of brain/evolve.py.

CPU tests pin the loaders to outputs of the reference's own Python functions
(tests/golden/evolve_golden.json, made by tests/golden/make_fixtures.py). The
GPU tests check that the in-process call equals the file-based CLI path that
brain/evolve.py:431-454 runs as a subprocess.
"""
import ctypes
import ctypes.util
import json
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "evolve_golden.json")) as f:
        return json.load(f)


def test_features_match_reference(golden):
    from codec_arena_gb300 import brain

    phi = brain.features(golden["genes"])
    assert phi.shape == (len(golden["genes"]), 166)
    np.testing.assert_array_equal(phi, np.asarray(golden["features"]))


def test_load_weights_migrations_match_reference(golden, tmp_path):
    from codec_arena_gb300 import brain

    for n, want in golden["load_weights"].items():
        p = tmp_path / f"w{n}.txt"
        brain.save_weights(str(p), [float(i) for i in range(int(n))])
        assert brain.load_weights(str(p)) == want


def test_genome_line_matches_reference(golden):
    from codec_arena_gb300 import brain

    for g, want in zip(golden["genes"], golden["genome_line"]):
        assert brain.genome_line({"id": 7, "gen": 3, "pa": 1, "pb": 2, "tribe": 5, "g": g}) == want


def _line(ntok_genes, rng):
    genes = rng.random(ntok_genes).round(4)
    return "9 2 3 4 5 " + " ".join(f"{x:.4f}" for x in genes)


@pytest.mark.parametrize("ng", [16, 22, 24, 27, 28, 29])
def test_load_pop_migration_agrees_with_genome_parse(tmp_path, ng):
    """evolve.py's load_pop and the screen's parseLine (with the v6 genes read)
    place every legacy gene in the same slot."""
    from codec_arena_gb300 import brain, genome

    rng = np.random.default_rng(ng)
    lines = [_line(ng, rng) for _ in range(5)]
    p = tmp_path / "pop.txt"
    p.write_text("# header\n\n" + "\n".join(lines) + "\n1 2 3\n")
    pop = brain.load_pop(str(p))
    assert len(pop) == 5
    for rec, line in zip(pop, lines):
        want = genome.parse_line(line, v6_fix=True)
        assert (rec["id"], rec["gen"], rec["pa"], rec["pb"], rec["tribe"]) == (9, 2, 3, 4, 5)
        np.testing.assert_array_equal(np.asarray(rec["g"], dtype=np.float32), want["g"])


def test_load_pop_seed_population():
    from codec_arena_gb300 import brain, genome

    path = os.path.join(GOLDEN, "pop_seed_96.txt")
    pop = brain.load_pop(path)
    assert len(pop) == 96
    el = genome.load_elites(path, v6_fix=True)
    np.testing.assert_array_equal(np.asarray([p["g"] for p in pop], dtype=np.float32), el["g"])
    # evolve.py writes elites back through genome_line: the text round trip is stable
    with open(path) as f:
        first = [ln.strip() for ln in f if ln.strip() and not ln.startswith("#")][0]
    assert brain.genome_line(pop[0]) == " ".join(first.split())


def test_sigma_text_to_f32_is_correctly_rounded():
    """The CLI reads --sigma with a correctly rounded decimal -> f32 parse; the
    in-process path goes decimal -> f64 -> f32. For every 4-decimal sigma in
    [0, 1] the two agree, so the in-process text round trip is exact."""
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.strtof.restype = ctypes.c_float
    libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    for i in range(10001):
        s = f"{i / 10000:.4f}"
        assert np.float32(float(s)) == np.float32(libc.strtof(s.encode(), None)), s


def test_next_population_ids():
    from codec_arena_gb300 import brain

    el = [{"id": i, "gen": 4, "pa": 0, "pb": 0, "tribe": 1, "g": [0.5] * 29} for i in range(3)]
    pr = [{"id": 0, "gen": 0, "pa": 10 + i, "pb": 20 + i, "tribe": i, "g": [0.25] * 29} for i in range(5)]
    nxt = brain.next_population(el, pr, shard=2, gen=3, pop=16, keep=4)
    assert [g["id"] for g in nxt] == [0, 1, 2, 20_000_051, 20_000_052, 20_000_053, 20_000_054]
    assert all(g["gen"] == 4 for g in nxt[3:]) and nxt[3]["pa"] == 10 and nxt[6]["pb"] == 23


def _evolve_elites(n=24):
    from codec_arena_gb300 import brain

    pop = brain.load_pop(os.path.join(GOLDEN, "pop_seed_96.txt"))
    for g in pop[:n]:
        g["gen"] = 6
    return pop[:n]


@pytest.mark.gpu
def test_in_process_equals_cli_files(csx, tmp_path):
    """screen_generation(text_roundtrip=True) returns exactly what evolve.py
    reads back from promoted.txt after the subprocess call."""
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import brain, cli, workloads as wl

    elites = _evolve_elites()
    seed, shard, gen, K, lam = 42, 3, 5, 96, 400_000
    el_path = tmp_path / "elites.txt"
    el_path.write_text("".join(brain.genome_line(g) + "\n" for g in elites))
    out, cnt = tmp_path / "promoted.txt", tmp_path / "screens.txt"
    rc = cli.main(["screen", "--model", wl.SURROGATE_161, "--elites", str(el_path), "--out", str(out),
                   "--count-out", str(cnt), "--lambda", str(lam), "--keep", str(K),
                   "--seed", str(seed * 1000003 + shard * 131 + gen), "--threads", "4",
                   "--sigma", f"{0.12 * (0.93 ** gen):.4f}", "--jump", "0.02", "--imm", "0.01"])
    assert rc == 0
    want = []
    for line in out.read_text().splitlines():
        t = line.split()
        if len(t) != 5 + brain.NG:
            continue
        want.append({"id": 0, "gen": 0, "pa": int(t[2]), "pb": int(t[3]), "tribe": int(t[4]),
                     "g": [float(x) for x in t[5:]]})
    got, screened = brain.screen_generation(elites, wl.surrogate_161(), screens=lam, keep=K, seed=seed,
                                            shard=shard, gen=gen, text_roundtrip=True)
    assert screened == int(cnt.read_text())
    assert len(want) == K and got == want


@pytest.mark.gpu
def test_in_process_direct_arrays(csx):
    """Without the text round trip the elites reach the GPU as f32 genes and
    the survivors keep their full f32 genes."""
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import brain, parallel, screen, workloads as wl

    elites = _evolve_elites()
    got, screened = brain.screen_generation(elites, wl.surrogate_161(), screens=300_000, keep=64, seed=9,
                                            shard=1, gen=2, sigma_decay=0.9)
    cfg = screen.Cfg(300_000, 64, parallel.island_seed(9, 1, 2), threads=4, sigma=0.12 * 0.9 ** 2)
    want, n = screen.screen(cfg, screen.Model.from_compact(wl.surrogate_161()), brain.elites_array(elites))
    assert screened == n == 300_000
    assert [p["pa"] for p in got] == want["pa"].tolist()
    np.testing.assert_array_equal(np.asarray([p["g"] for p in got], dtype=np.float32), want["g"])


def test_search_counter_bookkeeping(tmp_path):
    """screens_count.txt per shard, summed into the lifetime counters as
    tools/merge_results.py does (search_evals = evals + screens)."""
    from codec_arena_gb300 import brain

    for i, (ev, sc) in enumerate([(120, 2_650_000_000 * 20), (80, 10**9), (0, None)]):
        d = tmp_path / f"shard-{i}"
        d.mkdir()
        (d / "evals_count.txt").write_text(str(ev))
        if sc is not None:
            brain.write_screens_count(str(d), sc)
    assert (tmp_path / "shard-0" / "screens_count.txt").read_text() == str(53_000_000_000)
    st = brain.update_lifetime_counters(str(tmp_path), {"lifetime_evals": 99_950, "runs": 4, "milestones": {}})
    assert st["lifetime_evals"] == 100_150 and st["runs"] == 5
    assert st["search_evals"] == 99_950 + 200 + 54_000_000_000
    assert st["milestones"] == {"1e5": "run 5"}
    assert st["search_milestones"] == {"1e6": "run 5", "1e9": "run 5"}
    st2 = brain.update_lifetime_counters(str(tmp_path), st)
    assert st2["milestones"] == {"1e5": "run 5"} and st2["runs"] == 6


def test_extend_to_full_is_the_same_surface(orc):
    """A 166-coefficient model moved into the full layout scores every genome
    as the reference's Model.score surface does (16·w0 intercept), in FP64."""
    from codec_arena_gb300 import brain

    rng = np.random.default_rng(5)
    w = rng.normal(size=166).astype(np.float32)
    full = np.asarray(brain.extend_to_full(w), dtype=np.float64)
    assert full.shape == (465,)
    m = orc.model_from_compact(w)
    mf = orc.model_full_from_compact(full.astype(np.float32))
    for _ in range(10):
        g = rng.random(29).astype(np.float32)
        want = orc.score_f64(m, g)
        assert abs(float(brain.features_full(g)[0] @ full) - want) < 1e-9 * (1 + abs(want))
        assert abs(orc.score_f64(mf, g) - want) < 1e-9 * (1 + abs(want))


def test_load_weights_keeps_the_full_layout(tmp_path):
    from codec_arena_gb300 import brain

    w = [float(i) / 7 for i in range(465)]
    p = tmp_path / "w.txt"
    brain.save_weights(str(p), w)
    got = brain.load_weights(str(p))
    assert len(got) == 465 and np.allclose(got, w, rtol=1e-8)


@pytest.mark.gpu
def test_refit_surrogate_on_the_gpu(csx, tmp_path):
    """brain/evolve.py:250-268's semantics (False below 300 rows or for a
    prior of the wrong length) and its solution, for the 166 layout and the
    full 465 one, against the FP64 oracle."""
    import sys

    from conftest import ROOT, has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refit

    from codec_arena_gb300 import brain

    rng = np.random.default_rng(8)
    genes = rng.random((4000, 29)).astype(np.float32)
    fit = rng.normal(size=4000)
    rows = [(list(map(float, g)), float(f)) for g, f in zip(genes, fit)]
    out = tmp_path / "surrogate.txt"
    assert not brain.refit_surrogate(rows[:299], [0.0] * 166, str(out))
    assert not brain.refit_surrogate(rows, [0.0] * 153, str(out))
    for nf, full in ((166, False), (465, True)):
        prior = rng.normal(0, 0.1, nf)
        assert brain.refit_surrogate(rows, prior, str(out), alpha=50.0)
        got = np.asarray(brain.load_weights(str(out)))
        X = refit.features(genes, full=full)
        want = np.linalg.solve(X.T @ X + 50.0 * np.eye(nf), X.T @ fit + 50.0 * prior)
        # save_weights writes 9 significant digits
        np.testing.assert_allclose(got, want, rtol=2e-8, atol=1e-9 * np.abs(want).max())


@pytest.mark.gpu
def test_screen_generation_with_full_weights(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import brain, parallel, screen

    elites = _evolve_elites()
    w = np.random.default_rng(12).normal(0, 0.3, 465).astype(np.float32)
    got, n = brain.screen_generation(elites, w, screens=200_000, keep=32, seed=3, shard=0, gen=1)
    cfg = screen.Cfg(200_000, 32, parallel.island_seed(3, 0, 1), threads=4, sigma=0.12 * 0.93)
    want, m = screen.screen(cfg, screen.ModelFull.from_compact(w), brain.elites_array(elites))
    assert n == m == 200_000
    np.testing.assert_array_equal(np.asarray([p["g"] for p in got], dtype=np.float32), want["g"])
