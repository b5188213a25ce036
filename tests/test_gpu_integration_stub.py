"""The reference-side ctypes stub (codec_arena_gb300/evolve_binding.py, the
code INTEGRATION.md quotes) binds the library with ctypes alone and returns
what screen.screen returns."""
import importlib.util
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_integration_stub(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import _lib, brain, screen, workloads as wl

    os.environ["CSX_LIB"] = _lib.LIB_PATH
    spec = importlib.util.spec_from_file_location(
        "evolve_binding", os.path.join(ROOT, "codec_arena_gb300", "evolve_binding.py"))
    stub = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(stub)
    elites = brain.load_pop(os.path.join(ROOT, "tests", "golden", "pop_seed_96.txt"))[:20]
    w = [float(x) for x in wl.surrogate_161()]
    got, screened = stub.gpu_screen(w, elites, 200_000, 48, 11, 4, 0.1)
    want, n = screen.screen(screen.Cfg(200_000, 48, 11, threads=4, sigma=0.1),
                            screen.Model.from_compact(np.asarray(w, np.float32)), brain.elites_array(elites))
    assert screened == n == 200_000
    assert [(p["pa"], p["pb"], p["tribe"]) for p in got] == [(int(r["pa"]), int(r["pb"]), int(r["tribe"]))
                                                            for r in want]
    np.testing.assert_array_equal(np.asarray([p["g"] for p in got], np.float32), want["g"])
