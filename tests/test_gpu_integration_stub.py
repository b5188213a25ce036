"""The reference-side ctypes stub printed in INTEGRATION.md runs as written
(with the library path filled in) and returns what screen.screen returns."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_integration_stub(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import _lib, brain, screen, workloads as wl

    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text[text.index("### The reference-side ctypes stub"):]
    code = re.search(r"```python\n(.*?)```", sec, re.S).group(1)
    code = code.replace('"/path/to/codec_arena_gb300/libcsx_screen.so"', repr(_lib.LIB_PATH))
    ns = {}
    exec(compile(code, "INTEGRATION.md", "exec"), ns)
    elites = brain.load_pop(os.path.join(ROOT, "tests", "golden", "pop_seed_96.txt"))[:20]
    w = [float(x) for x in wl.surrogate_161()]
    got, screened = ns["gpu_screen"](w, elites, 200_000, 48, 11, 4, 0.1)
    want, n = screen.screen(screen.Cfg(200_000, 48, 11, threads=4, sigma=0.1),
                            screen.Model.from_compact(np.asarray(w, np.float32)), brain.elites_array(elites))
    assert screened == n == 200_000
    assert [(p["pa"], p["pb"], p["tribe"]) for p in got] == [(int(r["pa"]), int(r["pb"]), int(r["tribe"]))
                                                            for r in want]
    np.testing.assert_array_equal(np.asarray([p["g"] for p in got], np.float32), want["g"])
