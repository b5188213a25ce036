"""Multi-rank logic (gloo, world size 2): stream sharding of one generation and
island seeding, checked against the single-process oracle -- on CPU with the
oracle screening each rank's streams, and (GPU-marked) with the GPU engine
screening each rank's stream range."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT


def test_island_seed_matches_evolve():
    from codec_arena_gb300 import parallel

    # brain/evolve.py:437: --seed args.seed * 1000003 + args.shard * 131 + gen
    assert parallel.island_seed(42, 7, 3) == 42 * 1000003 + 7 * 131 + 3


def test_stream_ranges_cover_all_streams():
    from codec_arena_gb300 import parallel

    for T, lam, w in [(4, 10**9, 2), (4, 10**9, 3), (7, 100, 8), (100, 5, 2), (0, 10, 2)]:
        rs = parallel.stream_ranges(T, lam, w)
        flat = [t for r in rs for t in r]
        assert flat == list(range(max(1, min(T, lam))))


def test_merge_equals_single_process(orc):
    from codec_arena_gb300 import parallel, workloads as wl

    el = wl.seeded_elites(16, seed=3)
    m = orc.model_from_compact(wl.surrogate_161())
    lam, keep, T = 20_005, 50, 6
    c = orc.cfg(lam, keep, 9, threads=T)
    full, _ = orc.screen(c, m, el)
    parts = []
    for rg in parallel.stream_ranges(T, lam, 3):
        local = []
        for t in rg:
            my = lam - (T - 1) * (lam // T) if t == T - 1 else lam // T  # last stream: the remainder
            d = orc.stream_dump(c, m, el, t, my)
            d["index"] = np.arange(my)
            local.append(d)
        parts.append(parallel.merge_survivors(local, keep))
    assert parallel.merge_survivors(parts, keep).tobytes() == full.tobytes()


def _run_world_2(tmp_path, lam, keep, seed, T, engine, port, nproc=2):
    out = tmp_path / f"rank0_{engine}.json"
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={nproc}",
           "--master-addr=127.0.0.1", f"--master-port={port}",
           os.path.join(ROOT, "tests", "_dist_worker.py"), str(lam), str(keep), str(seed), str(T), str(out), engine]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.load(open(out))


@pytest.mark.gpu
def test_gloo_world_size_2_gpu_engine(orc, tmp_path):
    """Two ranks, each screening its stream range on the GPU, merged over gloo:
    equal to the oracle's single-process generation."""
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import _lib, workloads as wl

    lam, keep, seed, T = 3_000_001, 64, 8, 5
    res = _run_world_2(tmp_path, lam, keep, seed, T, "gpu", 29534)
    merged = np.frombuffer(bytes.fromhex(res["merged"]), dtype=_lib.SURVIVOR_DTYPE)
    full, _ = orc.screen(orc.cfg(lam, keep, seed, threads=T), orc.model_from_compact(wl.surrogate_161()),
                         wl.seeded_elites(16, seed=3))
    assert merged.tobytes() == full.tobytes()


def test_gloo_world_size_2(orc, tmp_path):
    from codec_arena_gb300 import _lib

    out = tmp_path / "rank0.json"
    lam, keep, seed, T = 12_000, 40, 5, 4
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=29533",
           os.path.join(ROOT, "tests", "_dist_worker.py"), str(lam), str(keep), str(seed), str(T), str(out)]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.load(open(out))
    assert res["world"] == 2 and res["slowest"] >= 1.0  # rank 1 adds 1 s: the max is taken
    merged = np.frombuffer(bytes.fromhex(res["merged"]), dtype=_lib.SURVIVOR_DTYPE)
    from codec_arena_gb300 import workloads as wl

    full, _ = orc.screen(orc.cfg(lam, keep, seed, threads=T), orc.model_from_compact(wl.surrogate_161()),
                         wl.seeded_elites(16, seed=3))
    assert merged.tobytes() == full.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("engine,nproc,T,port", [("items", 2, 4, 29541), ("items", 3, 2, 29542),
                                                 ("gpu", 3, 2, 29543)])
def test_gloo_split_one_generation_gpu(orc, tmp_path, engine, nproc, T, port):
    """One generation split over gloo ranks on the GPU: by work items (two
    ranks at T = 4; three ranks at T = 2, more ranks than streams) and by
    streams with three ranks at T = 2 (one rank has no stream and joins the
    gather empty). The merged survivors equal the oracle's single-process
    generation."""
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")
    from codec_arena_gb300 import _lib, workloads as wl

    lam, keep, seed = 2_000_003, 48, 13
    res = _run_world_2(tmp_path, lam, keep, seed, T, engine, port, nproc=nproc)
    merged = np.frombuffer(bytes.fromhex(res["merged"]), dtype=_lib.SURVIVOR_DTYPE)
    full, _ = orc.screen(orc.cfg(lam, keep, seed, threads=T), orc.model_from_compact(wl.surrogate_161()),
                         wl.seeded_elites(16, seed=3))
    assert merged.tobytes() == full.tobytes()


def test_gloo_more_ranks_than_streams_oracle(orc, tmp_path):
    """Three ranks at T = 2 with the oracle engine: the rank without a stream
    gathers an empty list and the merge equals the generation."""
    from codec_arena_gb300 import _lib, workloads as wl

    lam, keep, seed, T = 9_000, 30, 2, 2
    res = _run_world_2(tmp_path, lam, keep, seed, T, "oracle", 29544, nproc=3)
    merged = np.frombuffer(bytes.fromhex(res["merged"]), dtype=_lib.SURVIVOR_DTYPE)
    full, _ = orc.screen(orc.cfg(lam, keep, seed, threads=T), orc.model_from_compact(wl.surrogate_161()),
                         wl.seeded_elites(16, seed=3))
    assert res["world"] == 3 and merged.tobytes() == full.tobytes()
