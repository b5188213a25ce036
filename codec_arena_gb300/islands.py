"""Batched islands: several independent screens in one GPU pipeline.

An island is what one CI shard of the reference runs each generation
(brain/evolve.py with its own seed, elites and surrogate;
.github/workflows/arena.yml:56-92). `screen_batch` screens all islands in one
CUDA-graph launch of one pipeline and returns, per island, exactly what
`screen.screen` returns for that island alone. The islands' item building runs
on parallel streams; then, when every island's surrogate admits the pruning
bound and every island is large enough for pruning to pay (the library's
pruning floor), each island's pruning screen runs in turn over the whole GPU,
else one unpruned persistent screen kernel takes every island's candidates (a
FLAG_NO_PRUNE island selects that form for its batch). `Tune` holds the pipeline's tunables, which
change speed only; `autotune` picks them by timing.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import GENOME_DTYPE, SURVIVOR_DTYPE, check, lib
from .screen import Cfg, Model

MAX_ISLANDS = _lib.MAX_ISLANDS


@dataclass(frozen=True)
class Tune:
    item_cands: int = 0   # candidates per work item (0 = automatic)
    seg_cands: int = 0    # candidates per walk segment (0 = automatic)
    ctas_per_sm: int = 0  # persistent screen CTAs per SM (0 = as many as fit)

    def c(self) -> _lib.CsxBatchTune:
        return _lib.CsxBatchTune(int(self.item_cands), int(self.seg_cands), int(self.ctas_per_sm), 0)


def _pack(cfgs: Sequence[Cfg], models: Sequence[Model], elites: Sequence[np.ndarray]):
    n = len(cfgs)
    if not (len(models) == len(elites) == n):
        raise ValueError("cfgs, models and elites must have one entry per island")
    c_cfgs = (_lib.CsxCfg * n)(*[c.c() for c in cfgs])
    c_models = (_lib.CsxModel * n)(*[m.c for m in models])
    el = [np.ascontiguousarray(e) for e in elites]
    for e in el:
        if e.dtype != GENOME_DTYPE:
            raise TypeError("elites must be GENOME_DTYPE arrays")
    n_el = (ctypes.c_int * n)(*[int(e.shape[0]) for e in el])
    flat = np.concatenate(el) if el else np.zeros(0, GENOME_DTYPE)
    return c_cfgs, c_models, n_el, flat


def screen_batch(cfgs: Sequence[Cfg], models: Sequence[Model], elites: Sequence[np.ndarray],
                 tune: Optional[Tune] = None) -> List[Tuple[np.ndarray, int]]:
    """Screen every island in one graph launch: [(survivors, screened)] per island."""
    n = len(cfgs)
    c_cfgs, c_models, n_el, flat = _pack(cfgs, models, elites)
    keeps = [int(c.keep) for c in cfgs]
    out = np.zeros(max(1, sum(keeps)), dtype=SURVIVOR_DTYPE)
    n_out = (ctypes.c_uint64 * n)()
    scr = (ctypes.c_uint64 * n)()
    t = tune.c() if tune else None
    check(lib().csx_screen_batch(n, c_cfgs, c_models, flat.ctypes.data, n_el, ctypes.byref(t) if t else None,
                                 out.ctypes.data, n_out, scr), "screen_batch")
    res, off = [], 0
    for i in range(n):
        res.append((out[off: off + int(n_out[i])].copy(), int(scr[i])))
        off += keeps[i]
    return res


def screen_batch_device(cfgs: Sequence[Cfg], models: Sequence[Model], elites_dev, n_elites: Sequence[int],
                        out_dev, result_dev, tune: Optional[Tune] = None, stream=None) -> None:
    """Enqueue the batch on torch-owned device memory (no graph; capturable by
    the caller once a first call has sized the buffers).

    elites_dev: uint8 CUDA tensor of all islands' GENOME_DTYPE records back to
    back; out_dev: room for sum(keep) survivors (island i at sum of earlier
    keeps); result_dev: 4 int64 words per island (count, screened, error bits,
    items)."""
    import torch

    n = len(cfgs)
    c_cfgs = (_lib.CsxCfg * n)(*[c.c() for c in cfgs])
    c_models = (_lib.CsxModel * n)(*[m.c for m in models])
    n_el = (ctypes.c_int * n)(*[int(x) for x in n_elites])
    t = tune.c() if tune else None
    st = stream if stream is not None else torch.cuda.current_stream()
    check(lib().csx_screen_batch_device(n, c_cfgs, c_models, elites_dev.data_ptr(), n_el,
                                        ctypes.byref(t) if t else None, out_dev.data_ptr(), result_dev.data_ptr(),
                                        st.cuda_stream), "screen_batch_device")


def last_batch_info() -> dict:
    info = _lib.CsxBatchInfo()
    check(lib().csx_last_batch_info(ctypes.byref(info)))
    return {f: getattr(info, f) for f, _ in _lib.CsxBatchInfo._fields_}


__all__ = ["Tune", "screen_batch", "screen_batch_device", "last_batch_info", "MAX_ISLANDS"]
