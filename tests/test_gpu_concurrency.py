"""Concurrent use of the library: host threads calling the synchronous API at
once, and device-API calls on different CUDA streams sharing the per-device
scratch, must each return what a lone call returns."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")


def _cases():
    from codec_arena_gb300 import screen, workloads as wl

    m = screen.Model.from_compact(wl.surrogate_161())
    return [(screen.Cfg(200_000 + 37_000 * i, 32 + 8 * i, 100 + i, threads=1 + i % 5), m,
             wl.seeded_elites(8 + 9 * i, seed=20 + i)) for i in range(6)]


def test_host_threads_share_the_library():
    from codec_arena_gb300 import screen

    cases = _cases()
    want = [screen.screen(c, m, e) for c, m, e in cases]
    got = [None] * len(cases)
    errs = []

    def run(i):
        try:
            got[i] = screen.screen(*cases[i])
        except Exception as ex:  # surfaced below
            errs.append(ex)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(len(cases))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs, errs
    for (g, gn), (w, wn) in zip(got, want):
        assert gn == wn and g.tobytes() == w.tobytes()


def test_device_calls_on_two_streams():
    """Back-to-back device-API calls on different streams: the library orders
    them on its shared scratch, so each result equals its lone call."""
    import torch

    from codec_arena_gb300 import screen
    from codec_arena_gb300._lib import SURVIVOR_DTYPE

    cases = _cases()[:4]
    want = [screen.screen(c, m, e)[0] for c, m, e in cases]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    outs = []
    for i, (c, m, e) in enumerate(cases):
        d_el = torch.from_numpy(e.view(np.uint8).copy()).cuda()
        d_out = torch.zeros(c.keep * SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
        s = streams[i % 2]
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            screen.screen_device(c, m, d_el, d_out, d_res, stream=s)
        outs.append((d_el, d_out, d_res))
    torch.cuda.synchronize()
    for (d_el, d_out, d_res), w in zip(outs, want):
        res = d_res.cpu().numpy()
        assert res[2] == 0
        got = screen.survivors_from_bytes(d_out.cpu().numpy(), int(res[0]))
        assert got.tobytes() == w.tobytes()


def test_batch_and_single_interleaved():
    from codec_arena_gb300 import islands, screen

    cases = _cases()
    cfgs, models, elites = zip(*cases[:3])
    b1 = islands.screen_batch(cfgs, models, elites)
    s1 = screen.screen(*cases[4])
    b2 = islands.screen_batch(cfgs, models, elites)
    s2 = screen.screen(*cases[4])
    for (a, na), (b, nb) in zip(b1, b2):
        assert na == nb and a.tobytes() == b.tobytes()
    assert s1[0].tobytes() == s2[0].tobytes()
