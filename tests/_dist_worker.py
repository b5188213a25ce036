"""Worker for tests/test_parallel.py, launched by torch.distributed.run with
the gloo backend. Each rank screens its share of one generation's RNG streams
-- with the GPU engine (csx_screen_range) when the sixth argument is "gpu",
else with the CPU oracle -- then the ranks merge survivors over gloo and agree
on the slowest rank's time. With "items" each rank screens its share of the
generation's work items instead (csx_screen_items)."""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import numpy as np  # noqa: E402
import torch.distributed as dist  # noqa: E402

import oracle  # noqa: E402
from codec_arena_gb300 import parallel, workloads as wl  # noqa: E402


def main():
    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    lam, keep, seed, T = int(sys.argv[1]), int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4])
    out = sys.argv[5]
    engine = sys.argv[6] if len(sys.argv) > 6 else "oracle"
    el = wl.seeded_elites(16, seed=3)
    t0 = time.perf_counter()
    rg = parallel.stream_ranges(T, lam, world)[rank]
    if engine == "items":  # this rank's share of the generation's work items (csx_screen_items)
        from codec_arena_gb300 import screen

        mine, _ = screen.screen(screen.Cfg(lam, keep, seed, threads=T), screen.Model.from_compact(wl.surrogate_161()),
                                el, items=parallel.item_shard(rank, world))
    elif engine == "gpu":
        from codec_arena_gb300 import screen

        mine, _ = screen.screen(screen.Cfg(lam, keep, seed, threads=T), screen.Model.from_compact(wl.surrogate_161()),
                                el, streams=(rg.start, rg.stop))
    else:
        m = oracle.model_from_compact(wl.surrogate_161())
        c = oracle.cfg(lam, keep, seed, threads=T)
        Tn = max(1, min(T, lam))
        per = lam // Tn
        local = []
        for t in rg:
            my = lam - (Tn - 1) * per if t == Tn - 1 else per
            d = oracle.stream_dump(c, m, el, t, my)
            d["index"] = np.arange(my)
            local.append(d)
        mine = parallel.merge_survivors(local, keep)
    merged = parallel.gather_survivors(mine, keep)
    slowest = parallel.max_over_ranks(time.perf_counter() - t0 + rank)
    if rank == 0:
        with open(out, "w") as f:
            json.dump({"merged": merged.tobytes().hex(), "slowest": slowest, "world": world}, f)
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
