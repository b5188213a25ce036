"""Multi-process helpers for running screens on several GPUs.

The reference scales out by independent islands: every CI shard runs its own
generation loop with its own seed (brain/evolve.py:437, `seed * 1000003 +
shard * 131 + gen`) and the shards never exchange candidates
(.github/workflows/arena.yml:56-92). One island per rank therefore needs no
collective on the data path; ranks only agree on timing.

A single generation can also be split by RNG stream: streams are independent,
so each rank may screen a subset and the global top-K is the top-K of the
ranks' survivors under the reference's order (score descending, then stream,
then index). `merge_survivors` implements that merge.

torch.distributed is the transport (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

from typing import Iterable, List, Sequence

import numpy as np

from ._lib import SURVIVOR_DTYPE


def island_seed(seed: int, shard: int, gen: int = 0) -> int:
    """The screen seed of one shard's generation (brain/evolve.py:437)."""
    return int(seed) * 1000003 + int(shard) * 131 + int(gen)


def stream_ranges(threads: int, lam: int, world: int) -> List[range]:
    """Split the T = max(1, min(threads, lambda)) streams of one generation
    into `world` contiguous ranges (src/screen.zig:267). With more ranks than
    streams the last ranks get empty ranges (screen.screen returns no
    survivors for them, so they still join the gather); item_shard splits a
    generation over any number of ranks instead."""
    T = max(1, min(int(threads), int(lam)))
    base, extra = divmod(T, world)
    out, t0 = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append(range(t0, t0 + n))
        t0 += n
    return out


def item_shard(rank: int, world: int):
    """The items= argument of screen.screen for one rank's share of a
    generation's work items (csx_screen_items)."""
    return (int(rank), int(world))


def merge_survivors(parts: Iterable[np.ndarray], keep: int) -> np.ndarray:
    """Global top-`keep` of per-rank survivor lists (in rank order), in the
    reference's final order: score descending, then stream, then each list's
    own order. A stream lives in one rank's list when the generation is split
    by stream (that list already orders its exact ties as the reference's
    heap does), and in consecutive ranks' lists in index order when it is
    split by work items, so (rank, position) continues the order either way."""
    parts = [np.asarray(p, dtype=SURVIVOR_DTYPE) for p in parts]
    keys = [(np.full(len(p), r), np.arange(len(p))) for r, p in enumerate(parts)]
    if not any(len(p) for p in parts):
        return np.zeros(0, dtype=SURVIVOR_DTYPE)
    a = np.concatenate(parts)
    rank = np.concatenate([k[0] for k in keys])
    pos = np.concatenate([k[1] for k in keys])
    # NaN scores never survive (they have no order in the reference)
    ok = ~np.isnan(a["score"])
    a, rank, pos = a[ok], rank[ok], pos[ok]
    order = np.lexsort((pos, rank, a["stream"], -a["score"].astype(np.float64)))
    return a[order][: int(keep)]


def max_over_ranks(value: float, device=None) -> float:
    """Max of a per-rank float (timing) over the default process group."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_survivors(local: np.ndarray, keep: int, device=None) -> np.ndarray:
    """All ranks' survivor lists merged on every rank (fixed-size exchange of
    `keep` records per rank, padded with NaN scores)."""
    import torch
    import torch.distributed as dist

    local = np.asarray(local, dtype=SURVIVOR_DTYPE)
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return merge_survivors([local], keep)
    pad = np.zeros(int(keep), dtype=SURVIVOR_DTYPE)
    pad["score"] = np.nan
    pad[: len(local)] = local[:keep]
    raw = torch.from_numpy(pad.view(np.uint8).copy())
    if device is not None:
        raw = raw.to(device)
    bufs = [torch.empty_like(raw) for _ in range(dist.get_world_size())]
    dist.all_gather(bufs, raw)
    parts = [np.frombuffer(b.cpu().numpy().tobytes(), dtype=SURVIVOR_DTYPE) for b in bufs]
    return merge_survivors(parts, keep)


__all__ = ["island_seed", "stream_ranges", "item_shard", "merge_survivors", "max_over_ranks", "gather_survivors"]
