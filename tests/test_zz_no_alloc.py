"""csx_screen_device_noalloc against csx_screen_device (GPU, bit-exact).

The no-allocation entry point serves callers that cannot allocate device
memory: a process whose own memory pool owns the whole device, or one that
cannot afford the device-wide synchronisation cudaMalloc / cudaFree can bring
while its other streams run. Its scratch is a static array in the library that
every call shares, so two calls in a row with different configurations also
check that nothing from the first call leaks into the second.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(name, cfg, model, d_el, ne):
    import torch

    from codec_arena_gb300 import _lib, screen

    keep_n = min(cfg.keep, cfg.lambda_)
    d_out = torch.zeros(max(1, keep_n) * _lib.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    c = cfg.c()
    rc = getattr(_lib.lib(), name)(ctypes.byref(c), ctypes.byref(model.c), d_el.data_ptr(), ne,
                                   d_out.data_ptr(), keep_n, d_res.data_ptr(),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, (name, rc)
    torch.cuda.synchronize()
    res = d_res.cpu().numpy()
    return screen.survivors_from_bytes(d_out.cpu().numpy(), int(res[0])), res


def test_noalloc_equals_pooled_on_two_calls_in_a_row(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch

    from codec_arena_gb300 import screen, workloads as wl

    el = wl.seeded_elites(64)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    model = screen.Model.from_compact(wl.surrogate_161())
    cases = [screen.Cfg(3_000_000, 256, 7, threads=4),
             screen.Cfg(500_000, 100, 11, threads=7, imm_p=0.2, jump_p=0.1)]
    got = [_call("csx_screen_device_noalloc", c, model, d_el, len(el)) for c in cases]
    want = [_call("csx_screen_device", c, model, d_el, len(el)) for c in cases]
    for c, (g, gres), (w, wres) in zip(cases, got, want):
        assert gres[2] == 0 and wres[2] == 0
        assert gres[1] == wres[1] == c.lambda_
        assert len(g) == len(w) == min(c.keep, c.lambda_)
        assert g.tobytes() == w.tobytes()


def test_noalloc_rejects_oversized_configuration(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch

    from codec_arena_gb300 import _lib, screen, workloads as wl

    el = wl.seeded_elites(8)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    model = screen.Model.from_compact(wl.surrogate_161())
    cfg = screen.Cfg(10**12, 64, 1, threads=4)
    d_out = torch.zeros(64 * _lib.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    c = cfg.c()
    rc = _lib.lib().csx_screen_device_noalloc(ctypes.byref(c), ctypes.byref(model.c), d_el.data_ptr(),
                                              len(el), d_out.data_ptr(), 64, d_res.data_ptr(), None)
    assert rc == _lib.ERR_LIMIT


def test_noalloc_bench_generation_fits_and_equals(csx):
    """The bench generation (2.65e9 candidates, T = 4, top 256) fits the static
    scratch and equals csx_screen_device; so does a generation whose streams
    hold many walk segments with mixed immigrant and jump probabilities."""
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch

    from codec_arena_gb300 import screen, workloads as wl

    el = wl.seeded_elites(64)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    model = screen.Model.from_compact(wl.surrogate_161())
    for c in (screen.Cfg(2_650_000_000, 256, 7, threads=4),
              screen.Cfg(200_000_000, 64, 3, threads=2, imm_p=0.2, jump_p=0.1)):
        g, gres = _call("csx_screen_device_noalloc", c, model, d_el, len(el))
        w, wres = _call("csx_screen_device", c, model, d_el, len(el))
        assert gres[2] == 0 and gres[1] == c.lambda_
        assert g.tobytes() == w.tobytes()


def test_noalloc_refuses_precision_flags(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch

    from codec_arena_gb300 import _lib, screen, workloads as wl

    el = wl.seeded_elites(8)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    model = screen.Model.from_compact(wl.surrogate_161())
    d_out = torch.zeros(16 * _lib.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    for flag in (_lib.FLAG_TC_BF16, _lib.FLAG_TC_FP16):
        c = screen.Cfg(10_000, 16, 1, threads=4, flags=flag).c()
        rc = _lib.lib().csx_screen_device_noalloc(ctypes.byref(c), ctypes.byref(model.c), d_el.data_ptr(),
                                                  len(el), d_out.data_ptr(), 16, d_res.data_ptr(), None)
        assert rc == _lib.ERR_BAD_ARGS
