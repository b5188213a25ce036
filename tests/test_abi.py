"""C ABI of libcsx_screen.so without a GPU: exports, struct layout, and the
host-side functions (model layout, parsing, formatting, CLI argument errors)
against the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu

HEADERS = [os.path.join(ROOT, "include", h) for h in ("csx_screen.h", "csx_surrogate.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"\b(csx_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_expected_api():
    names = declared_functions()
    for must in ("csx_screen", "csx_screen_device", "csx_model_from_compact", "csx_model_parse",
                 "csx_genome_parse_line", "csx_elites_parse", "csx_screen_cli", "csx_strerror"):
        assert must in names


def test_library_exports_every_declared_symbol(csx):
    for name in declared_functions():
        assert hasattr(csx, name), name
    from codec_arena_gb300 import _lib

    assert set(declared_functions()) == set(_lib.SIGNATURES)
    assert csx.csx_abi_version() == 1


def test_struct_layout_matches_oracle():
    import oracle
    from codec_arena_gb300 import _lib

    assert _lib.GENOME_DTYPE == oracle.GENOME_DTYPE
    assert _lib.SURVIVOR_DTYPE == oracle.SURVIVOR_DTYPE
    assert ctypes.sizeof(_lib.CsxCfg) == ctypes.sizeof(oracle.OrcCfg)
    assert ctypes.sizeof(_lib.CsxModel) == ctypes.sizeof(oracle.OrcModel)


def test_cfg_defaults(csx):
    from codec_arena_gb300 import _lib

    c = _lib.CsxCfg()
    csx.csx_cfg_default(ctypes.byref(c))
    assert (c.lambda_, c.keep, c.seed, c.threads) == (1000000, 192, 42, 4)
    assert (c.sigma, c.jump_p, c.imm_p) == (np.float32(0.12), np.float32(0.02), np.float32(0.01))


@pytest.mark.parametrize("n", [153, 159, 161, 164, 165, 166])
def test_model_from_compact_matches_oracle(csx, orc, n):
    from codec_arena_gb300.screen import Model

    w = np.random.default_rng(n).normal(size=n).astype(np.float32)
    got = Model.from_compact(w)
    want = orc.model_from_compact(w)
    assert got.w0 == want.w0
    np.testing.assert_array_equal(got.w_lin, np.ctypeslib.as_array(want.w_lin))
    np.testing.assert_array_equal(got.w_quad, np.ctypeslib.as_array(want.w_quad))


def test_model_from_compact_bad_size(csx):
    from codec_arena_gb300 import CsxError
    from codec_arena_gb300.screen import Model

    with pytest.raises(CsxError) as e:
        Model.from_compact(np.zeros(160, np.float32))
    assert e.value.status == -1


def _random_line(rng, ntok):
    toks = [str(rng.integers(0, 2**40)), str(rng.integers(0, 100)), str(rng.integers(0, 9999)),
            str(rng.integers(0, 9999)), str(rng.integers(0, 12))]
    for _ in range(ntok - 5):
        x = rng.random()
        toks.append(rng.choice([f"{x:.4f}", f"{x:.8e}", f"{x * 3 - 1:.6f}", "0", "1", "-0.0000"]))
    return rng.choice([" ", "\t", "  "]).join(toks)


@pytest.mark.parametrize("flags", [0, 4])
def test_parse_line_matches_oracle(csx, orc, flags):
    from codec_arena_gb300 import genome

    rng = np.random.default_rng(7 + flags)
    for _ in range(300):
        ntok = int(rng.choice([21, 27, 29, 32, 33, 34, 20, 30, 35]))
        line = _random_line(rng, ntok)
        try:
            want = orc.parse_line(line, flags)
            werr = None
        except ValueError:
            werr = True
        if werr:
            with pytest.raises(Exception):
                genome.parse_line(line, v6_fix=bool(flags))
            continue
        got = genome.parse_line(line, v6_fix=bool(flags))
        if want is None:
            assert got is None
        else:
            assert got.tobytes() == want.tobytes(), line


@pytest.mark.parametrize("tok", ["1_000", "+5", "-0", "-5", "_1", "1_", "0x10", "", "12a"])
def test_parse_int_forms(csx, orc, tok):
    from codec_arena_gb300 import genome

    line = f"{tok} 0 0 0 1 " + " ".join(["0.5"] * 16)
    try:
        want = orc.parse_line(line)
    except ValueError:
        want = "err"
    try:
        got = genome.parse_line(line)
    except Exception:
        got = "err"
    if isinstance(want, str) or want is None:
        assert (got == want) if isinstance(got, str) or got is None else False
    else:
        assert got.tobytes() == want.tobytes()


def test_elites_text_matches_oracle(csx, orc):
    from codec_arena_gb300 import genome, workloads

    text = open(os.path.join(workloads.GOLDEN_DIR, "pop_seed_96.txt")).read()
    for v6 in (False, True):
        got = genome.load_elites_text(text, v6_fix=v6)
        want = orc.elites_parse(text, 4 if v6 else 0)
        assert len(got) == 96
        assert got.tobytes() == want.tobytes()
    # as written, the 34-token seed lines lose genes 16..21
    assert np.all(genome.load_elites_text(text)["g"][:, 16:22] == 0)


def test_model_parse_matches_oracle(csx, orc):
    from codec_arena_gb300 import screen, workloads

    text = open(workloads.SURROGATE_161).read()
    np.testing.assert_array_equal(screen.parse_model_text(text), orc.model_parse(text))
    m = screen.load_model(workloads.SURROGATE_161)
    assert m.w0 == np.float32(-28.108021)


def test_format_lines(csx):
    from codec_arena_gb300 import _lib, genome, screen

    g = genome.make_genomes(np.linspace(0, 1, 29, dtype=np.float32)[None, :], ids=[77], tribes=[5])[0]
    line = genome.format_line(g)
    assert len(line.split()) == 34 and line.startswith("77 0 0 0 5 0.0000")
    back = genome.parse_line(line, v6_fix=True)
    np.testing.assert_allclose(back["g"], g["g"], atol=1e-4)
    s = np.zeros(1, dtype=_lib.SURVIVOR_DTYPE)
    s["pa"], s["pb"], s["tribe"] = 3, 4, 2
    s["g"] = np.arange(29, dtype=np.float32) / 29
    l34 = screen.format_survivor(s[0])
    l29 = screen.format_survivor(s[0], _lib.FLAG_OUTPUT_29)
    assert l34.endswith("\n") and len(l34.split()) == 34 and l34.startswith("0 0 3 4 2 0.0000 0.0345")
    assert len(l29.split()) == 29


def _cli(args):
    from codec_arena_gb300 import cli

    return cli.main(["screen", *args])


def test_cli_errors_before_gpu(csx, tmp_path, capfd):
    from codec_arena_gb300 import workloads

    model = workloads.SURROGATE_161
    one = tmp_path / "one.txt"
    one.write_text("0 0 0 0 1 " + " ".join(["0.5"] * 29) + "\n")
    bad = tmp_path / "bad.txt"
    bad.write_text("160 " + " 0" * 160)
    assert _cli(["--model", str(tmp_path / "missing.txt")]) == 1
    assert _cli(["--model", str(bad), "--elites", str(one)]) == 1
    assert "BadModel" in capfd.readouterr().err
    assert _cli(["--model", model, "--elites", str(one)]) == 1
    assert "NeedTwoElites" in capfd.readouterr().err
    assert _cli(["--model", model, "--lambda"]) == 1
    assert "BadArgs" in capfd.readouterr().err
    assert _cli(["--model", model, "--lambda", "12x"]) == 1


@pytest.mark.skipif(has_gpu(), reason="checks the no-device status")
def test_screen_without_device_fails_loudly(csx):
    from codec_arena_gb300 import CsxError, screen, workloads

    m = screen.Model.from_compact(workloads.seeded_normal_model())
    with pytest.raises(CsxError) as e:
        screen.screen(screen.Cfg(1000, 10, 1), m, workloads.seeded_elites(8))
    assert e.value.status == -8


def test_screen_argument_checks(csx):
    from codec_arena_gb300 import CsxError, screen, workloads

    m = screen.Model.from_compact(workloads.seeded_normal_model())
    el = workloads.seeded_elites(8)
    with pytest.raises(CsxError) as e:
        screen.screen(screen.Cfg(1000, 10, 1), m, el[:1])
    assert e.value.status == -2
    with pytest.raises(CsxError) as e:
        screen.screen(screen.Cfg(1000, 0, 1), m, el)
    assert e.value.status == -3
    with pytest.raises(CsxError) as e:
        screen.screen(screen.Cfg(1000, 5000, 1), m, el)
    assert e.value.status == -6
