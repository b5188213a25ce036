"""Autotuner selection and cache logic with a fake timer (no GPU)."""
import json

from codec_arena_gb300 import autotune, screen
from codec_arena_gb300.islands import Tune


def test_pick_lowest_median():
    times = {Tune(): [5.0, 9.0, 9.0, 9.0], Tune(ctas_per_sm=2): [1.0, 4.0, 3.0, 100.0], Tune(item_cands=64): [2, 6, 6, 6]}
    it = {k: iter(v) for k, v in times.items()}
    best, table = autotune.pick(lambda t: next(it[t]), list(times), reps=3)
    assert best == Tune(ctas_per_sm=2)
    assert dict(table)[Tune(ctas_per_sm=2)] == 4.0


def test_cache_roundtrip(tmp_path, monkeypatch):
    import numpy as np

    from codec_arena_gb300 import workloads as wl

    monkeypatch.setenv("CSX_TUNE_CACHE", str(tmp_path / "t.json"))
    cfgs = [screen.Cfg(1000, 8, 1), screen.Cfg(2000, 8, 2)]
    el = [wl.seeded_elites(4), wl.seeded_elites(5)]
    calls = []

    def timer(t):
        calls.append(t)
        return 1.0 + t.ctas_per_sm

    best, _ = autotune.autotune(cfgs, [None, None], el, candidates=[Tune(ctas_per_sm=2), Tune(ctas_per_sm=1)],
                                reps=1, timer=timer, device_name="fake")
    assert best == Tune(ctas_per_sm=1) and len(calls) == 4
    best2, _ = autotune.autotune(cfgs, [None, None], el, candidates=[Tune(ctas_per_sm=2)], timer=timer,
                                 device_name="fake")
    assert best2 == best and len(calls) == 4  # cached: no timing
    d = json.load(open(tmp_path / "t.json"))
    assert len(d) == 1
    k = autotune.shape_key(cfgs, [4, 5], "fake")
    assert k in d and autotune.shape_key(cfgs, [4, 6], "fake") != k
