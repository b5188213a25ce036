"""Autotuner for the batched-islands pipeline.

The pipeline's tunables (work-item size, walk-segment size, persistent CTAs
per SM) change how the work is cut, never the survivors. `autotune` times a
list of candidate settings on the actual batch (optionally with every budget
scaled down), keeps the fastest and caches it per batch shape in a JSON file
(CSX_TUNE_CACHE, default ~/.cache/codec_arena_gb300/tune.json).
"""
from __future__ import annotations

import hashlib
import json
import os
import statistics
from typing import Callable, Dict, List, Optional, Sequence, Tuple

from .islands import Tune

CANDIDATES: List[Tune] = [
    Tune(),                                   # automatic: 3 CTAs/SM, ~8 items per thread, 32768-candidate segments
    Tune(ctas_per_sm=2),
    Tune(item_cands=1024),
    Tune(item_cands=4096),
    Tune(seg_cands=8192),
    Tune(seg_cands=8192, item_cands=1024),
    Tune(seg_cands=131072),
]


def cache_path() -> str:
    return os.environ.get("CSX_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "codec_arena_gb300", "tune.json"))


def shape_key(cfgs, n_elites: Sequence[int], device_name: str = "") -> str:
    """Batch shape: per island (lambda to 3 significant digits, keep, threads,
    elites), plus the device name."""
    parts = [device_name] + [f"{float(c.lambda_):.3g}/{c.keep}/{c.threads}/{int(ne)}" for c, ne in zip(cfgs, n_elites)]
    return hashlib.sha1("|".join(parts).encode()).hexdigest()[:16]


def _load(path: str) -> Dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, key: str, entry: Dict) -> None:
    d = _load(path)
    d[key] = entry
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def pick(timer: Callable[[Tune], float], candidates: Sequence[Tune] = CANDIDATES, reps: int = 3
         ) -> Tuple[Tune, List[Tuple[Tune, float]]]:
    """Time every candidate `reps` times (after one untimed call each) and
    return the one with the lowest median, with the table."""
    table = []
    for t in candidates:
        timer(t)
        ms = statistics.median(timer(t) for _ in range(max(1, reps)))
        table.append((t, ms))
    best = min(table, key=lambda x: x[1])[0]
    return best, table


def gpu_timer(cfgs, models, elites) -> Callable[[Tune], float]:
    """A timer running the batch on the current CUDA device (CUDA events on
    the current stream), inputs resident."""
    import numpy as np
    import torch

    from . import islands
    from ._lib import SURVIVOR_DTYPE

    flat = np.concatenate([np.ascontiguousarray(e) for e in elites])
    d_el = torch.from_numpy(flat.view(np.uint8).copy()).cuda()
    n_el = [int(e.shape[0]) for e in elites]
    d_out = torch.empty(sum(int(c.keep) for c in cfgs) * SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.empty(4 * len(cfgs), dtype=torch.int64, device="cuda")

    def run(t: Tune) -> float:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        islands.screen_batch_device(cfgs, models, d_el, n_el, d_out, d_res, tune=t)
        b.record()
        b.synchronize()
        return a.elapsed_time(b)

    return run


def autotune(cfgs, models, elites, candidates: Sequence[Tune] = CANDIDATES, reps: int = 3, scale: float = 1.0,
             timer: Optional[Callable[[Tune], float]] = None, use_cache: bool = True, device_name: str = ""
             ) -> Tuple[Tune, List[Tuple[Tune, float]]]:
    """Pick the fastest Tune for this batch shape (cached). `scale` < 1 times
    a copy of the batch with every budget scaled down."""
    from dataclasses import replace

    n_el = [int(e.shape[0]) for e in elites]
    if not device_name:
        try:
            import torch

            device_name = torch.cuda.get_device_name() if torch.cuda.is_available() else ""
        except Exception:
            device_name = ""
    key = shape_key(cfgs, n_el, device_name)
    path = cache_path()
    if use_cache:
        hit = _load(path).get(key)
        if hit:
            return Tune(*hit["tune"]), [(Tune(*t), ms) for t, ms in hit["table"]]
    if timer is None:
        tcfgs = [replace(c, lambda_=max(1, int(c.lambda_ * scale))) for c in cfgs] if scale != 1.0 else list(cfgs)
        timer = gpu_timer(tcfgs, models, elites)
    best, table = pick(timer, candidates, reps)
    if use_cache:
        _store(path, key, {"tune": [best.item_cands, best.seg_cands, best.ctas_per_sm],
                           "table": [[[t.item_cands, t.seg_cands, t.ctas_per_sm], ms] for t, ms in table]})
    return best, table


__all__ = ["CANDIDATES", "autotune", "pick", "shape_key", "gpu_timer", "cache_path"]
