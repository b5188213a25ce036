#!/usr/bin/env python3
"""Benchmark of the GB300 screen funnel (candidates/s on one generation).

Workload (one "step" = one generation's screen): 2.65e9 candidates, 64 seeded
elites, the reference's committed v3 surrogate (161 coefficients), top 256,
T = 4 splitmix64 streams (the reference CI's --threads), sigma 0.12, jump
0.02, immigrants 0.01, seed 7. Synthetic seeded inputs; no dataset.

  value  device-resident: elites on the GPU, survivors stay on the GPU; CUDA
         events on the launch stream around each step; L2 flushed between steps
  e2e    the same metric through the C ABI's host-buffer call (csx_screen):
         H2D of the elites and D2H of the survivors inside the timed region
  roofline  the persistent screen kernel against the measured splitmix64 and
         integer-issue rates of this GPU (the path is integer-issue bound)
  cpu_baseline  the C restatement of the Zig screen (oracle/) on this host's
         cores, T = 4 as the reference CI, on a bounded prefix sample
  precision_forms  the same generation with the quadratic block on the tensor
         cores (BF16, and FP16 with x' = 2g - 1): throughput beside the plain
         FP32 value, top-256 recall against the FP64 top-256, score errors

The metric names the BF16 tensor-core form against the plain FP32 form; the
line's value is the plain FP32 fused screen (the reference's own f32
semantics, bit-exact), and precision_forms carries the BF16 / FP16 values.
`--workload precision` prints a line whose value is the BF16 form;
`--workload islands` the batched-islands workload, `--workload refit` the
GPU ridge refit and the surrogate's forward / backward kernels (with the full
29-gene surface's refit beside it), `--workload full` the generation screened
on the full 29-gene quadratic surface.

`--impl reference` times the reference's CPU implementation of the path (the
restatement: Zig is not available) on the same workload, rank 0 only.
N > 1 GPUs run independent islands (one seed each, like the reference's CI
shards): weak scaling, no collective on the data path.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LAMBDA = 2_650_000_000
KEEP = 256
THREADS = 4
SEED = 7
N_ELITES = 64
# Algorithmic 32-bit lane-ops per candidate of the full synthesis and score
# (the unpruned form's count, and the cost of each candidate queued for the
# reference order): 61.75 splitmix64 draws x 20 + 29 genes x 5 + the score's
# FMA x 2 = 1760 with a linear tail (weights on genes 16..28). Without one (the
# committed v3 and the 153-term layouts) the score needs genes 0..15 only: the
# tail's 0.99 x 26 crossover draws and 0.01 x 13 immigrant draws (x 20) and its
# 13 genes (x 5) and 13 FMA (x 2) drop out: 1151.6.
def full_synth_ops(tail):
    if tail:
        return 1760.0
    return 1760.0 - (0.99 * 26 + 0.01 * 13) * 20 - 13 * (5 + 2)


# The pruning form per candidate: the header's 4 draws (parents, immigrant
# test, jump test) + 0.02 jump index draws, the 16 crossover-bit draws of the
# 0.99 crossover candidates (x 20 lane-ops each), the bound's FP32 work on them
# (4 x 16 lane-ops beside the tensor core's 16 x 16 MACs, 8 packs), and the
# full synthesis for the fraction q queued for the reference-order score.
PRUNE_DRAWS = 4.02 + 0.99 * 16
PRUNE_FIXED_OPS = PRUNE_DRAWS * 20 + 0.99 * (4 * 16 + 8)
PRUNE_TC_FLOP = 0.99 * 2 * 16 * 16  # tensor-core flops per candidate (the bound's gradient)


def prune_ops(q, tail):
    return PRUNE_FIXED_OPS + q * full_synth_ops(tail)


def has_tail(model):
    """Whether a surface (screen.Model) carries a linear weight on genes 16..28."""
    return any(x != 0.0 for x in model.c.w_lin[16:29])


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--lambda", dest="lam", type=int, default=LAMBDA)
    ap.add_argument("--threads", type=int, default=THREADS)
    ap.add_argument("--keep", type=int, default=KEEP)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-precision", action="store_true", help="skip the tensor-core precision forms")
    ap.add_argument("--workload", default="generation",
                    choices=["generation", "islands", "precision", "refit", "full", "config1"],
                    help="islands: 20 islands batched in one graph launch (not the headline line); "
                         "config1: the reference workload's first configuration (lambda 1e6, top 32, "
                         "seeded 153-term surface)")
    ap.add_argument("--split", default="islands", choices=["islands", "items"],
                    help="N > 1 GPUs: one island per rank (weak scaling), or one generation split by work "
                         "items across the ranks with a survivor gather (strong scaling)")
    ap.add_argument("--islands", type=int, default=20)
    ap.add_argument("--no-autotune", action="store_true", help="islands: the automatic tunables, no tuning runs")
    ap.add_argument("--islands-scale", type=float, default=1.0,
                    help="scale every island budget (small cases for profiling)")
    return ap.parse_args(argv)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


def _config1_args(args):
    """The reference workload's first configuration: lambda 1e6, top 32."""
    args.lam, args.keep = 1_000_000, 32


def workload_config(args, n):
    if args.workload == "config1":
        return {"workload": f"the reference workload's first configuration: lambda={args.lam} candidates, "
                            f"{N_ELITES} elites drawn from seed 1, 153-coefficient surface drawn N(0,1) x 0.1 "
                            f"from seed 2, top-{args.keep}, T={args.threads} RNG streams",
                "lambda": args.lam, "keep": args.keep, "threads": args.threads, "elites": N_ELITES,
                "surrogate": "seeded N(0,1) x 0.1, 153 coefficients (v1 layout), seed 2", "sigma": 0.12,
                "jump_p": 0.02, "imm_p": 0.01, "seed": SEED,
                "l2": "flushed between steps (256 MiB write)", "parallelism": "single"}
    return {"workload": f"screen generation: lambda={args.lam} candidates, {N_ELITES} seeded elites, "
                        f"committed v3 surrogate (161 coefficients), top-{args.keep}, "
                        f"T={args.threads} RNG streams" + (f", {n} islands" if n > 1 else ""),
            "lambda": args.lam, "keep": args.keep, "threads": args.threads, "elites": N_ELITES,
            "surrogate": "state/surrogate.txt (v3, 161)", "sigma": 0.12, "jump_p": 0.02, "imm_p": 0.01,
            "seed": SEED, "l2": "flushed between steps (256 MiB write); inputs are a 10 KB elite pool",
            "parallelism": f"islands{n}" if n > 1 else "single"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_index):
        self.dev = dev_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()),
                                   default=None)}


def cpu_baseline(args, seconds):
    """The oracle (C restatement of src/screen.zig) at T streams, T threads, on a
    prefix sample of the workload sized to about `seconds` of CPU time."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    from codec_arena_gb300 import workloads as wl

    el = wl.seeded_elites(N_ELITES)
    m = oracle.model_from_compact(wl.surrogate_161())
    T = args.threads
    lam = 400_000
    t0 = time.perf_counter()
    oracle.screen(oracle.cfg(lam, args.keep, SEED, threads=T), m, el, cpu_threads=T)
    dt = time.perf_counter() - t0
    lam = int(min(args.lam, max(lam, lam * seconds / max(dt, 1e-6))))
    lam -= lam % T
    t0 = time.perf_counter()
    _, screened = oracle.screen(oracle.cfg(lam, args.keep, SEED, threads=T), m, el, cpu_threads=T)
    dt = time.perf_counter() - t0
    out = {"value": screened / dt, "unit": "candidates/s", "cores": T, "kind": "port",
           "sample": f"first {lam // T} candidates of each of the T={T} streams "
                     f"({lam} candidates, {dt:.1f} s), C restatement built -O3 -ffp-contract=off",
           "host_threads_available": os.cpu_count()}
    # every host core: one stream per core (T is part of a screen's identity, so this
    # is the same budget split into more streams)
    n = os.cpu_count() or T
    if n > T:
        lam_all = int(min(args.lam, lam * n / T))
        lam_all -= lam_all % n
        t0 = time.perf_counter()
        _, scr = oracle.screen(oracle.cfg(lam_all, args.keep, SEED, threads=n), m, el, cpu_threads=n)
        dt = time.perf_counter() - t0
        out["all_cores"] = {"value": scr / dt, "cores": n, "streams": n,
                            "sample": f"{lam_all} candidates as T={n} streams on {n} threads ({dt:.1f} s)"}
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    steps, warm = args.steps, args.warmup
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    from codec_arena_gb300 import workloads as wl

    if args.workload == "config1":
        _config1_args(args)
    el = wl.seeded_elites(N_ELITES)
    w = wl.seeded_normal_model(seed=2) if args.workload == "config1" else wl.surrogate_161()
    m = oracle.model_from_compact(w)
    T = args.threads
    # bounded sample per step: the T-stream prefix that takes ~2 s on T threads
    lam = 400_000
    t0 = time.perf_counter()
    oracle.screen(oracle.cfg(lam, args.keep, SEED, threads=T), m, el, cpu_threads=T)
    dt = time.perf_counter() - t0
    lam = int(min(args.lam, max(lam, lam * 2.0 / max(dt, 1e-6))))
    lam -= lam % T
    for _ in range(warm):
        oracle.screen(oracle.cfg(lam // 10, args.keep, SEED, threads=T), m, el, cpu_threads=T)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        oracle.screen(oracle.cfg(lam, args.keep, SEED, threads=T), m, el, cpu_threads=T)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    v = lam * steps / tot
    line = {"impl": "reference", "metric": METRIC,
            "value": v, "unit": "candidates/s", "n_gpus": world, "steps": steps, "warmup": warm,
            "ms_per_step": 1000 * tot / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": v / PUBLISHED_CAND_S, "vs_baseline_source": PUBLISHED_SOURCE,
            "dtype": "u64/f32", "data": "synthetic (seeded)",
            "config": dict(workload_config(args, 1),
                           sample=f"each timed step screens the first {lam // T} candidates of each of the "
                                  f"T={T} streams ({lam} of the {args.lam} candidates; a stream's content does "
                                  "not depend on lambda, so the rate is the generation's); ms_per_step is that "
                                  "sample's time"),
            "cpu_baseline": {"value": v, "unit": "candidates/s", "cores": T, "kind": "port",
                             "sample": f"each step: first {lam // T} candidates of each of T={T} "
                                       f"streams ({lam} candidates) on {T} threads; Zig is not "
                                       "available, the C restatement of src/screen.zig runs"},
            "e2e": {"value": v, "unit": "candidates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_islands(args):
    """Batched islands: `args.islands` islands (budgets log-uniform in [1e8,
    2.65e9], 16..256 elites, own seeded N(0, 0.1) 153-term surfaces, top-K in
    {32, 128, 256}, T = 4) screened by one graph launch of the batch pipeline
    per step, tunables from the autotuner. Reported beside the same islands
    run as separate single-island screens."""
    import numpy as np
    import torch

    from codec_arena_gb300 import autotune, islands, screen, workloads as wl

    torch.cuda.set_device(0)
    isl = wl.seeded_islands(args.islands)
    cfgs = [screen.Cfg(max(1, int(d["lambda"] * args.islands_scale)), d["keep"], d["seed"], threads=d["threads"])
            for d in isl]
    models = [screen.Model.from_compact(d["weights"]) for d in isl]
    elites = [d["elites"] for d in isl]
    total = sum(c.lambda_ for c in cfgs)
    t0 = time.perf_counter()
    # tuned on the batch itself (full budgets) over the plausible settings
    cands = [islands.Tune(), islands.Tune(ctas_per_sm=2), islands.Tune(seg_cands=131072)]
    if args.no_autotune:
        best, table = islands.Tune(), []
    else:
        best, table = autotune.autotune(cfgs, models, elites, candidates=cands, scale=1.0, reps=1)
    tune_s = time.perf_counter() - t0
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(max(3, args.warmup)):
        islands.screen_batch(cfgs, models, elites, tune=best)
    sampler = ClockSampler(0)
    sampler.start()
    dev_ms, wall = [], []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = islands.screen_batch(cfgs, models, elites, tune=best)
        wall.append(time.perf_counter() - t)
        dev_ms.append(islands.last_batch_info()["ms_device"])
    clocks = sampler.stop()
    info = islands.last_batch_info()
    assert all(n == c.lambda_ for (_, n), c in zip(res, cfgs))
    # the same islands as separate screens (device API, CUDA events)
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    seq_ms = 0.0
    for c, m, e in zip(cfgs, models, elites):
        d_el = torch.from_numpy(e.view(np.uint8).copy()).cuda()
        d_out = torch.zeros(c.keep * 168, dtype=torch.uint8, device="cuda")
        screen.screen_device(c, m, d_el, d_out, d_res)
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        screen.screen_device(c, m, d_el, d_out, d_res)
        b.record()
        b.synchronize()
        seq_ms += a.elapsed_time(b)
    ms = statistics.mean(dev_ms)
    line = {"metric": "candidates/sec (batched islands, 1 GB300)", "value": total / (ms / 1000.0),
            "unit": "candidates/s", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64/f32", "data": "synthetic (seeded)",
            "config": {"workload": f"{len(cfgs)} islands in one graph launch: budgets log-uniform 1e8..2.65e9 "
                                   f"(total {total}), 16..256 seeded elites, seeded N(0,0.1) 153-term surfaces, "
                                   "top-K in {32,128,256}, T=4",
                       "islands": [[c.lambda_, c.keep, int(e.shape[0])] for c, e in zip(cfgs, elites)],
                       "l2": "flushed between steps (256 MiB write)"},
            "e2e": {"value": total / statistics.mean(wall), "unit": "candidates/s",
                    "h2d_bytes_per_step": int(sum(e.nbytes for e in elites)),
                    "d2h_bytes_per_step": int(sum(len(r[0]) for r in res) * 168),
                    "api": "csx_screen_batch (host buffers; capture/update + graph launch + copies)"},
            "sequential_single_screens": {"ms": seq_ms, "value": total / (seq_ms / 1000.0)},
            "tune": {"chosen": [best.item_cands, best.seg_cands, best.ctas_per_sm], "tuning_s": tune_s,
                     "table_ms": [[[t.item_cands, t.seg_cands, t.ctas_per_sm], ms_] for t, ms_ in table]},
            "graph": info, "clocks": clocks, "gpu_launches": int(info["launches"]) * args.steps}
    print(json.dumps(line), flush=True)


def _fp64_scores(model, g):
    import numpy as np

    g = np.asarray(g, dtype=np.float64)
    L = np.tril(model.w_quad.astype(np.float64).reshape(16, 16))
    return 16 * float(model.w0) + g @ model.w_lin.astype(np.float64) + np.einsum("ni,ij,nj->n", g[:, :16], L, g[:, :16])


METRIC = "candidates/sec, 1 GB300: BF16-TC fused vs FP32 plain at top-256 recall>=0.999"
# The reference's own published screen throughput: its Zig SIMD kernel, 4 threads
PUBLISHED_CAND_S = 17.2e6
PUBLISHED_SOURCE = "17.2 M candidates/s, Zig SIMD screen, 4 threads (docs/SCALE.md:26)"


def _profile_summary() -> dict:
    """ncu figures of the default screen kernel kept under profiles/ (DRAM
    traffic per launch scaled to the full workload, pipe utilisation)."""
    try:
        with open(os.path.join(ROOT, "profiles", "screen_pt_kernel_ncu.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def hbm_ceiling(traffic_bytes, ms):
    """DRAM bytes of one launch over its time, against the measured HBM copy
    bandwidth (MEASURED_PEAKS.json hbm_gbs; else the 6.8 TB/s fallback)."""
    pk = _measured_peaks().get("hbm_gbs")
    src = "MEASURED_PEAKS.json hbm_gbs" if pk else "fallback 6.8 TB/s"
    pk = pk or 6800.0
    if not traffic_bytes or not ms:
        return {"achieved": None, "peak": pk, "unit": "GB/s", "frac": None, "peak_source": src}
    gbs = traffic_bytes / (ms * 1e-3) / 1e9
    return {"achieved": gbs, "peak": pk, "unit": "GB/s", "frac": gbs / pk, "peak_source": src}


def issue_slots(achieved_tops, clocks):
    """The algorithmic lane-ops/s against the GPU's instruction issue limit:
    one warp instruction per scheduler per clock, 4 schedulers per SM, at the
    SM clock sampled during the timed region (its maximum if none)."""
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not mhz:
        return {"achieved": achieved_tops, "peak": None, "unit": "Tlane-op/s", "frac": None}
    peak = 4 * 32 * sms * mhz * 1e6 / 1e12
    return {"achieved": achieved_tops, "peak": peak, "unit": "Tlane-op/s", "frac": achieved_tops / peak,
            "peak_source": f"issue limit: 4 schedulers x 32 lanes x {sms} SMs x {mhz:.0f} MHz"}


FORMS = (
    ("fp32_unpruned", "FLAG_NO_PRUNE", "every candidate synthesised and scored (FFMA filter, reference f32 "
                                       "order near the threshold): the plain FP32 form"),
    ("fp32_prune_ffma", "FLAG_PRUNE_FFMA", "pruning, the bound's gradient by FP32 FMA; reference f32 order"),
    ("bf16_tc", "FLAG_TC_BF16", "precision form: pruning bound on BF16 tensor cores, queued candidates "
                                "filtered by FFMA and scored in FP64, survivors the FP64 top-K"),
    ("fp16_tc", "FLAG_TC_FP16", "precision form as bf16_tc with FP16 tiles"),
    ("bf16_tc_unpruned", "FLAG_TC_BF16|FLAG_NO_PRUNE", "precision form without pruning: the quadratic "
                                                        "block of every candidate on BF16 tensor cores, an "
                                                        "FP64 band"),
)


def precision_forms(args, default=None):
    """The generation in each form beside the default (pruned, FP16 tensor-core
    bound, reference f32 order): throughput (CUDA events, L2 flushed), screen
    kernel time, candidates rescored, top-K recall against the FP64 top-K,
    and the tensor-core scores' errors against FP64."""
    import numpy as np
    import torch

    from codec_arena_gb300 import _lib, precision, screen, workloads as wl

    el = wl.seeded_elites(N_ELITES)
    model = screen.Model.from_compact(wl.surrogate_161())
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out = {}
    forms = list(FORMS)
    if default is None:
        forms.insert(0, ("fp32_prune_tc", "", "default: pruning, the bound's gradient on FP16 tensor cores"))
    for name, flagnames, what in forms:
        flag = 0
        for fn in filter(None, flagnames.split("|")):
            flag |= getattr(_lib, fn)
        cfg = screen.Cfg(args.lam, args.keep, SEED, threads=args.threads, flags=flag | _lib.FLAG_STAGE_TIMES)
        d_out = torch.zeros(args.keep * 168, dtype=torch.uint8, device="cuda")
        d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
        for _ in range(max(3, args.warmup)):
            screen.screen_device(cfg, model, d_el, d_out, d_res)
        ms, kms = [], []
        for _ in range(args.steps):
            flush.fill_(1)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            screen.screen_device(cfg, model, d_el, d_out, d_res)
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
            kms.append(screen.last_run_info()["ms_screen"])
        res = d_res.cpu().numpy()
        assert res[2] == 0 and res[1] == args.lam
        info = screen.last_run_info()
        out[name] = {"form": what, "flags": flagnames or "0", "value": args.lam / (statistics.mean(ms) / 1000),
                     "ms_per_step": statistics.mean(ms), "screen_kernel_ms": statistics.mean(kms),
                     "rescored": info["exact_evals"], "screen_ctas": info["screen_ctas"],
                     "_surv": screen.survivors_from_bytes(d_out.cpu().numpy(), int(res[0]))}
        if "TC" in flagnames:
            # tensor work: pruned forms 2 x 16 x 16 flop per crossover candidate (the bound's
            # gradient), the unpruned form one 128x16x16 MMA per 128 candidates (512 flop)
            flop = 512.0 if "NO_PRUNE" in flagnames else PRUNE_TC_FLOP
            tf = flop * args.lam / (statistics.mean(kms) * 1e-3) / 1e12
            pk = _measured_peaks().get("bf16_tflops") or 1900.0
            out[name]["tensor_roofline"] = {"achieved": tf, "peak": pk, "unit": "TFLOP/s", "frac": tf / pk,
                                            "note": "the tensor cores carry a 16x16 product per candidate; "
                                                    "the form stays bound by the integer synthesis"}
    if default is not None:
        v, ms_step, kms_, rescored, surv = default
        out["fp32_prune_tc"] = {"form": "default: pruning, the bound's gradient on FP16 tensor cores (the line's "
                                        "value)", "flags": "0", "value": v, "ms_per_step": ms_step,
                                "screen_kernel_ms": kms_, "rescored": rescored, "_surv": surv}
    # FP64 ground truth: the exact screen's top 4096 rescored in FP64, certified complete below
    big, _ = screen.screen(screen.Cfg(args.lam, 4096, SEED, threads=args.threads), model, el)
    s64 = _fp64_scores(model, big["g"])
    order = np.lexsort((big["index"], big["stream"], -s64))
    K = args.keep
    truth = {(int(big["stream"][i]), int(big["index"][i])) for i in order[:K]}
    L = np.tril(model.w_quad.reshape(16, 16).astype(np.float64))
    A = 16 * abs(float(model.w0)) + np.abs(model.w_lin).sum() + np.abs(L).sum()
    e32 = 36 * 2.0 ** -24 * A  # the exact order's FP32 error bound (gamma_35 of the absolute terms)
    certified = bool(float(big["score"][-1]) + e32 < s64[order[K - 1]])
    ref = out["fp32_prune_tc"]["_surv"].tobytes()
    for name in out:
        sv = out[name].pop("_surv")
        have = {(int(r["stream"]), int(r["index"])) for r in sv}
        out[name]["recall_vs_fp64"] = len(have & truth) / K
        if name.startswith("fp32"):
            out[name]["identical_to_default"] = sv.tobytes() == ref
    g_top = torch.from_numpy(np.ascontiguousarray(big["g"])).cuda()
    rng = np.random.default_rng(5)
    g_rand = rng.random((1_000_000, 29), dtype=np.float32)
    s64_rand = _fp64_scores(model, g_rand)
    g_rand = torch.from_numpy(g_rand).cuda()
    for form in ("bf16", "fp16"):
        # the tensor-core score (csx_tc_score, the unpruned precision form's) against FP64
        e_top = np.abs(precision.tc_score(model, g_top, form).cpu().numpy() - s64)
        e_rand = np.abs(precision.tc_score(model, g_rand, form).cpu().numpy() - s64_rand)
        out[form + "_tc"]["tc_score_error_vs_fp64"] = {
            "max_abs_top4096": float(e_top.max()), "mean_abs_top4096": float(e_top.mean()),
            "max_rel_top4096": float((e_top / np.abs(s64)).max()),
            "max_abs_uniform1e6": float(e_rand.max()), "mean_abs_uniform1e6": float(e_rand.mean())}
    return {"forms": out, "fp64_truth": {"from": "exact FP32 screen top-4096 rescored in FP64",
                                         "certified_complete": certified}}


def run_precision(args):
    """`--workload precision`: the BF16 tensor-core form as the line's value."""
    import torch

    torch.cuda.set_device(0)
    sampler = ClockSampler(0)
    sampler.start()
    p = precision_forms(args)
    clocks = sampler.stop()
    f = p["forms"]
    line = {"metric": METRIC, "value": f["bf16_tc"]["value"], "unit": "candidates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": f["bf16_tc"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": f["bf16_tc"]["value"] / PUBLISHED_CAND_S,
            "vs_baseline_source": PUBLISHED_SOURCE,
            "dtype": "bf16 tensor cores (pruning bound) + f64 ranking; genes u64/f32", "data": "synthetic (seeded)",
            "config": workload_config(args, 1),
            "bf16_over_fp32": f["bf16_tc"]["value"] / f["fp32_unpruned"]["value"],
            "bf16_over_fp32_pruned": f["bf16_tc"]["value"] / f["fp32_prune_tc"]["value"],
            "clocks": clocks}
    line.update(p)
    print(json.dumps(line), flush=True)


def run_refit(args):
    """Differentiable refit: ridge refit (alpha 1e-2) of 400,000 rows x 16 genes
    (seeded quadratic truth + Student-t(3) noise) on the GPU -- FP64 normal
    equations and FP64 Cholesky -- beside the reference's own numpy FP64 refit
    (brain/evolve.py:259-265) on the host cores; the surrogate's forward and
    backward kernels over the same rows."""
    import numpy as np
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refit as orc_refit

    from codec_arena_gb300 import build, surrogate, workloads as wl

    torch.cuda.set_device(0)
    genes, fit, w_true = wl.refit_table()
    n, nf, alpha = genes.shape[0], 153, 1e-2
    d_g, d_y = torch.from_numpy(genes).cuda(), torch.from_numpy(fit).cuda()
    prior = torch.zeros(nf, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(fn):
        out = []
        for _ in range(max(3, args.warmup)):
            fn()
        for _ in range(args.steps):
            flush.fill_(1)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            out.append(a.elapsed_time(b))
        return statistics.mean(out)

    sampler = ClockSampler(0)
    sampler.start()
    ms_refit = timed(lambda: surrogate.refit(d_g, d_y, prior, alpha))
    ms_gram = timed(lambda: surrogate.normal_equations(d_g, d_y, nf))
    G, r = surrogate.normal_equations(d_g, d_y, nf)
    ms_solve = timed(lambda: surrogate.ridge_solve(G, r, alpha, prior))
    coef = torch.from_numpy(w_true.astype(np.float32)).cuda().requires_grad_(True)
    gg = d_g.clone().requires_grad_(True)
    ms_fwd = timed(lambda: surrogate.score(d_g, coef.detach()))
    ms_fwd_bwd = timed(lambda: surrogate.score(gg, coef).sum().backward())
    clocks = sampler.stop()
    w = surrogate.refit(d_g, d_y, prior, alpha).cpu().numpy()
    # the reference's refit on the host (numpy FP64)
    t0 = time.perf_counter()
    w_np = orc_refit.refit_solve(genes, fit, np.zeros(nf), alpha)
    cpu_s = time.perf_counter() - t0
    bench = ctypes.CDLL(build.BENCH_LIB)
    bench.csx_bench_issue_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    dfma = ctypes.c_double(0)
    bench.csx_bench_issue_rate(4, ctypes.byref(dfma))
    gram_flop = 2.0 * n * (nf * (nf + 1) / 2 + nf)  # upper triangle + right-hand side, FP64
    line = {"metric": "ridge refit time (400,000 rows x 16 genes, alpha 1e-2, FP64), 1 GB300", "value": ms_refit,
            "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_refit,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64 (normal equations, "
            "Cholesky); f32 genes", "data": "synthetic (seeded quadratic truth + 0.5 * Student-t(3) noise)",
            "config": {"workload": "ridge refit toward a zero prior: 400,000 rows of 16 genes, 153 features, alpha 1e-2",
                       "rows": n, "features": nf, "alpha": alpha, "l2": "flushed between steps (256 MiB write)"},
            "stages_ms": {"normal_equations": ms_gram, "cholesky_solve": ms_solve},
            "roofline": {"bound": "fp64", "kernel": "sg_gram_kernel", "achieved": gram_flop / (ms_gram * 1e-3) / 1e12,
                         "peak": 2 * dfma.value / 1e12, "unit": "TFLOP/s",
                         "frac": gram_flop / (ms_gram * 1e-3) / (2 * dfma.value) if dfma.value else None,
                         "peak_source": "measured: DFMA issue rate of this GPU (csx_bench_issue_rate kind 4)"},
            "vs_numpy_fp64": {"max_abs_diff": float(np.abs(w - w_np).max()), "max_abs_w": float(np.abs(w_np).max()),
                              "numpy_seconds": cpu_s, "host_threads": os.cpu_count(),
                              "speedup": cpu_s * 1000 / ms_refit},
            "surrogate_rows_per_s": {"forward": n / (ms_fwd * 1e-3), "forward_backward": n / (ms_fwd_bwd * 1e-3)},
            "clocks": clocks, "gpu_launches": 4 * args.steps}
    line["full_surface"] = refit_full(args, timed, dfma.value)
    print(json.dumps(line), flush=True)


def refit_full(args, timed, dfma):
    """The same refit on the full surface: 400,000 rows of 29 genes, 465
    features (all pairs), against numpy FP64 on the host."""
    import numpy as np
    import torch

    import refit as orc_refit

    from codec_arena_gb300 import surrogate, workloads as wl

    genes, fit, w_true = wl.refit_table_full()
    n, nf, alpha = genes.shape[0], 465, 1e-2
    d_g, d_y = torch.from_numpy(genes).cuda(), torch.from_numpy(fit).cuda()
    prior = torch.zeros(nf, dtype=torch.float64, device="cuda")
    ms_refit = timed(lambda: surrogate.refit(d_g, d_y, prior, alpha))
    ms_gram = timed(lambda: surrogate.normal_equations(d_g, d_y, nf))
    G, r = surrogate.normal_equations(d_g, d_y, nf)
    ms_solve = timed(lambda: surrogate.ridge_solve(G, r, alpha, prior))
    w = surrogate.refit(d_g, d_y, prior, alpha).cpu().numpy()
    t0 = time.perf_counter()
    w_np = orc_refit.refit_solve(genes, fit, np.zeros(nf), alpha)
    cpu_s = time.perf_counter() - t0
    gram_flop = 2.0 * n * (nf * (nf + 1) / 2 + nf)
    return {"rows": n, "features": nf, "alpha": alpha, "ms": ms_refit,
            "stages_ms": {"normal_equations": ms_gram, "cholesky_solve": ms_solve},
            "roofline": {"bound": "fp64", "kernel": "sg_gram_kernel", "achieved": gram_flop / (ms_gram * 1e-3) / 1e12,
                         "peak": 2 * dfma / 1e12, "unit": "TFLOP/s",
                         "frac": gram_flop / (ms_gram * 1e-3) / (2 * dfma) if dfma else None},
            "vs_numpy_fp64": {"max_abs_diff": float(np.abs(w - w_np).max()), "max_abs_w": float(np.abs(w_np).max()),
                              "numpy_seconds": cpu_s, "speedup": cpu_s * 1000 / ms_refit},
            "max_abs_err_vs_truth": float(np.abs(w - w_true).max())}


def run_full(args):
    """`--workload full`: the generation workload screened on the full
    quadratic surface (all 29 genes; the committed v3 surrogate moved into the
    465-coefficient layout, new pairs 0): candidates/s by CUDA events, L2
    flushed between steps, and the issue roofline at its algorithmic work
    (1235 RNG + 145 gene + 2 x 464 FMA lane-ops per candidate)."""
    import numpy as np
    import torch

    from codec_arena_gb300 import _lib, brain, screen, workloads as wl

    torch.cuda.set_device(0)
    el = wl.seeded_elites(N_ELITES)
    model = screen.ModelFull.from_compact(
        np.asarray(brain.extend_to_full(brain.migrate_weights(wl.surrogate_161())), dtype=np.float32))
    cfg = screen.Cfg(args.lam, args.keep, SEED, threads=args.threads, flags=_lib.FLAG_STAGE_TIMES)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    d_out = torch.zeros(args.keep * _lib.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(max(3, args.warmup)):
        screen.screen_device(cfg, model, d_el, d_out, d_res)
    torch.cuda.synchronize()
    res = d_res.cpu().numpy()
    assert res[2] == 0 and res[1] == args.lam, f"device result {res}"
    sampler = ClockSampler(0)
    sampler.start()
    ms, kms = [], []
    for _ in range(args.steps):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        screen.screen_device(cfg, model, d_el, d_out, d_res)
        b.record()
        b.synchronize()
        ms.append(a.elapsed_time(b))
        kms.append(screen.last_run_info()["ms_screen"])
    clocks = sampler.stop()
    info = screen.last_run_info()
    ops = 1235 + 145 + 2 * 464
    achieved = args.lam / (statistics.mean(kms) * 1e-3) * ops / 1e12
    line = {"metric": "candidates/sec, full 29-gene quadratic surface, 1 GB300", "value":
            args.lam / (statistics.mean(ms) / 1000), "unit": "candidates/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": statistics.mean(ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64/f32", "data": "synthetic (seeded)",
            "config": dict(workload_config(args, 1), surrogate="state/surrogate.txt (v3, 161) in the full "
                           "465-coefficient layout, new pairs 0"),
            "roofline": dict(issue_slots(achieved, clocks), kernel="csx::screen_kernel<true, FullScreenArgs>",
                             algorithmic_ops_per_candidate=ops, bound="int/fp32-issue"),
            "stages_ms_last_step": {k: round(v, 4) for k, v in info.items() if k.startswith("ms_")},
            "clocks": clocks, "gpu_launches": int(info["launches"]) * args.steps}
    print(json.dumps(line), flush=True)


def run_config1(args):
    """`--workload config1`: the reference workload's first configuration
    (lambda 1e6, top 32, 64 elites from seed 1, the seeded 153-term surface)
    through the same pipeline, the device-resident value and the host-buffer
    e2e, beside the oracle on the host cores."""
    import numpy as np
    import torch

    from codec_arena_gb300 import _lib, screen, workloads as wl

    _config1_args(args)
    torch.cuda.set_device(0)
    el = wl.seeded_elites(N_ELITES, seed=1)
    w = wl.seeded_normal_model(seed=2)
    model = screen.Model.from_compact(w)
    cfg = screen.Cfg(args.lam, args.keep, SEED, threads=args.threads, flags=_lib.FLAG_STAGE_TIMES)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    d_out = torch.zeros(args.keep * _lib.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(max(3, args.warmup)):
        screen.screen_device(cfg, model, d_el, d_out, d_res)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    ms = []
    for _ in range(args.steps):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        screen.screen_device(cfg, model, d_el, d_out, d_res)
        b.record()
        b.synchronize()
        ms.append(a.elapsed_time(b))
    clocks = sampler.stop()
    res = d_res.cpu().numpy()
    assert res[2] == 0 and res[1] == args.lam, f"device result {res}"
    info = screen.last_run_info()
    hcfg = screen.Cfg(args.lam, args.keep, SEED, threads=args.threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        surv, _ = screen.screen(hcfg, model, el)
    e2e_t = (time.perf_counter() - t0) / args.steps
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    t0 = time.perf_counter()
    want, _ = oracle.screen(oracle.cfg(args.lam, args.keep, SEED, threads=args.threads),
                            oracle.model_from_compact(w), el, cpu_threads=args.threads)
    cpu_s = time.perf_counter() - t0
    value = args.lam / (statistics.mean(ms) / 1000.0)
    line = {"metric": METRIC, "value": value, "unit": "candidates/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": statistics.mean(ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": value / PUBLISHED_CAND_S, "vs_baseline_source": PUBLISHED_SOURCE,
            "dtype": "u64/f32", "data": "synthetic (seeded)", "config": workload_config(args, 1),
            "e2e": {"value": args.lam / e2e_t, "unit": "candidates/s", "h2d_bytes_per_step": int(el.nbytes),
                    "d2h_bytes_per_step": int(len(surv) * _lib.SURVIVOR_DTYPE.itemsize + 32),
                    "api": "csx_screen (host buffers, synchronous)"},
            "identical_to_oracle": surv.tobytes() == want.tobytes(),
            "stages_ms_last_step": {k: round(v, 4) for k, v in info.items() if k.startswith("ms_")},
            "cpu_baseline": {"value": args.lam / cpu_s, "unit": "candidates/s", "cores": args.threads,
                             "kind": "port", "sample": f"the whole configuration ({args.lam} candidates, "
                                                       f"{cpu_s:.2f} s) on {args.threads} threads"},
            "clocks": clocks, "gpu_launches": int(info["launches"]) * args.steps}
    print(json.dumps(line), flush=True)


def run_split_items(args):
    """`--split items` on N GPUs: ONE generation (the default workload) split
    across the ranks by work items (csx_screen_items), the ranks' survivors
    gathered and merged (parallel.gather_survivors): strong scaling. Each step
    is the host-buffer call plus the gather, timed on the host around a
    barrier, the max over ranks."""
    import numpy as np
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from codec_arena_gb300 import parallel, screen, workloads as wl

    el = wl.seeded_elites(N_ELITES)
    model = screen.Model.from_compact(wl.surrogate_161())
    cfg = screen.Cfg(args.lam, args.keep, SEED, threads=args.threads)

    def step():
        mine, n = screen.screen(cfg, model, el, items=parallel.item_shard(rank, world))
        return parallel.gather_survivors(mine, args.keep, device="cuda"), n

    for _ in range(max(3, args.warmup)):
        merged, _ = step()
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    scr = 0
    for _ in range(args.steps):
        merged, n = step()
        scr += n
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    dt = parallel.max_over_ranks(time.perf_counter() - t0, device="cuda")
    clocks = sampler.stop()
    total = parallel.max_over_ranks(float(scr), device="cuda")  # per rank: its share's count
    if rank != 0:
        return
    value = args.lam * args.steps / dt
    line = {"metric": METRIC, "value": value, "unit": "candidates/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": value / PUBLISHED_CAND_S, "vs_baseline_source": PUBLISHED_SOURCE,
            "dtype": "u64/f32", "data": "synthetic (seeded)",
            "config": dict(workload_config(args, 1), parallelism=f"items{world}",
                           split="one generation split by work items across the ranks, survivors gathered"),
            "e2e": {"value": value, "unit": "candidates/s", "h2d_bytes_per_step": int(el.nbytes),
                    "d2h_bytes_per_step": int(args.keep * 168),
                    "api": "csx_screen_items (host buffers) + gather_survivors, every step"},
            "best_score": float(merged["score"][0]) if len(merged) else None,
            "largest_share_screened": total / args.steps, "clocks": clocks}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "config1" and args.impl != "reference":
        return run_config1(args)
    if args.split == "items" and args.impl != "reference" and args.workload == "generation":
        return run_split_items(args)
    if args.workload == "refit" and args.impl != "reference":
        return run_refit(args)
    if args.workload == "full" and args.impl != "reference":
        return run_full(args)
    if args.workload == "precision" and args.impl != "reference":
        return run_precision(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "islands":
        return run_islands(args)
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from codec_arena_gb300 import _lib, build, screen, workloads as wl

    build.build()
    bench = ctypes.CDLL(build.BENCH_LIB)
    bench.csx_bench_issue_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]

    el = wl.seeded_elites(N_ELITES)
    model = screen.Model.from_compact(wl.surrogate_161())
    from codec_arena_gb300 import parallel

    seed = SEED if world == 1 else parallel.island_seed(SEED, rank)  # one island per rank
    cfg = screen.Cfg(args.lam, args.keep, seed, threads=args.threads, flags=_lib.FLAG_STAGE_TIMES)
    d_el = torch.from_numpy(el.view(np.uint8).copy()).cuda()
    d_out = torch.zeros(args.keep * _lib.SURVIVOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_res = torch.zeros(4, dtype=torch.int64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream()

    def step():
        screen.screen_device(cfg, model, d_el, d_out, d_res, stream=st)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    res = d_res.cpu().numpy()
    assert res[2] == 0 and res[1] == args.lam, f"device result {res}"

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    sampler = ClockSampler(local)
    sampler.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    screen_ms, stage = [], []
    barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        ev[i][0].record(st)
        step()
        ev[i][1].record(st)
        info = screen.last_run_info()  # waits for this step's last stage
        screen_ms.append(info["ms_screen"])
        stage.append(info)
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - w0
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = sum(step_ms) / 1000.0
    t_dev = parallel.max_over_ranks(t_dev, device="cuda")
    value = world * args.lam * args.steps / t_dev
    launches = stage[-1]["launches"]

    # e2e: host buffers through the C ABI (H2D elites, D2H survivors timed)
    e2e_steps = max(1, min(3, args.steps))
    hcfg = screen.Cfg(args.lam, args.keep, seed, threads=args.threads)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        surv, scr = screen.screen(hcfg, model, el)
    e2e_t = time.perf_counter() - t0
    e2e_t = parallel.max_over_ranks(e2e_t, device="cuda")
    e2e = {"value": world * args.lam * e2e_steps / e2e_t, "unit": "candidates/s",
           "h2d_bytes_per_step": int(el.nbytes + ctypes.sizeof(_lib.CsxModel) + ctypes.sizeof(_lib.CsxCfg)),
           "d2h_bytes_per_step": int(len(surv) * _lib.SURVIVOR_DTYPE.itemsize + 32),
           "api": "csx_screen (host buffers, synchronous)"}

    if rank != 0:
        return
    rates = {}
    for kind, name in ((0, "int_alu"), (1, "imad"), (2, "ffma"), (3, "splitmix64")):
        r = ctypes.c_double(0)
        if bench.csx_bench_issue_rate(kind, ctypes.byref(r)) == 0:
            rates[name] = r.value
    ms_screen = statistics.mean(screen_ms)
    cand_s_kernel = args.lam / (ms_screen / 1000.0)
    q = statistics.mean(st["exact_evals"] for st in stage) / args.lam  # queued for the reference order
    tail = has_tail(model)
    ops = prune_ops(q, tail)
    achieved = cand_s_kernel * ops / 1e12
    slots = issue_slots(achieved, clocks)
    prof = _profile_summary()
    traffic = prof.get("bytes_per_launch_full_workload") if args.lam == LAMBDA else None
    tc_tf = cand_s_kernel * PRUNE_TC_FLOP / 1e12
    bf16_peak = _measured_peaks().get("bf16_tflops")
    roofline = {
        "bound": "int-issue", "kernel": prof.get("kernel", "csx::screen_pt_kernel<16, true, false>"),
        "achieved": achieved, "peak": slots["peak"], "unit": "Tlane-op/s", "frac": slots["frac"],
        "peak_source": slots.get("peak_source"),
        "algorithmic_ops_per_candidate": ops,
        "ops_model": ("pruning form: %.2f draws x 20 lane-ops (4 header draws, 0.02 jump index, 16 crossover "
                      "bits for the 0.99 crossover candidates) + 0.99 x 72 bound lane-ops + q x %.1f for the "
                      "fraction q queued for the synthesis and reference-order score (measured q; %s)"
                      % (PRUNE_DRAWS, full_synth_ops(tail),
                         "genes 0..28" if tail else "genes 0..15: the surface has no linear weight past gene 15")),
        "queued_fraction": q,
        "traffic": traffic,
        "traffic_source": prof.get("traffic_note"),
        "kernel_ms_per_launch": ms_screen,
        "ncu": prof.get("ncu"),
        "issue_rates_measured": rates,
        "alu_probe_frac": (achieved / (rates["int_alu"] / 1e12)) if rates.get("int_alu") else None,
        # the other two ceilings: HBM (the launch's DRAM traffic against the
        # measured copy bandwidth) and the tensor pipe (the bound's gradient:
        # 2 x 16 x 16 flop per crossover candidate)
        "hbm": hbm_ceiling(traffic, ms_screen),
        "tensor": {"achieved": tc_tf, "unit": "TFLOP/s", "peak": bf16_peak,
                   "frac": tc_tf / bf16_peak if bf16_peak else None,
                   "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)"},
    }
    line = {"metric": METRIC, "value": value, "unit": "candidates/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": 1000.0 * t_dev / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": value / PUBLISHED_CAND_S, "vs_baseline_source": PUBLISHED_SOURCE,
            "dtype": "u64/f32", "data": "synthetic (seeded)",
            "config": workload_config(args, world), "e2e": e2e, "roofline": roofline,
            "clocks": clocks, "gpu_launches": int(launches * args.steps),
            "stages_ms_last_step": {k: round(v, 4) for k, v in stage[-1].items() if k.startswith("ms_")},
            "shape": dict({k: stage[-1][k] for k in ("screen_ctas", "segments", "seg_draws", "item_cands")},
                          items=int(res[3])),
            "exact_evals_last_step": stage[-1]["exact_evals"],
            "form": "pruning screen: bound's gradient on the FP16 tensor cores, survivors in the reference's "
                    "f32 order (byte-identical to the unpruned screen)",
            "wall_s": wall}
    if world == 1 and not args.no_precision:
        # the other forms of the same generation beside this value: unpruned
        # FP32, the FFMA bound, and the BF16 / FP16 precision forms
        line["precision_forms"] = precision_forms(
            args, default=(value, line["ms_per_step"], ms_screen, stage[-1]["exact_evals"],
                           screen.survivors_from_bytes(d_out.cpu().numpy(), int(d_res[0].item()))))
        f = line["precision_forms"]["forms"]
        line["bf16_over_fp32"] = f["bf16_tc"]["value"] / f["fp32_unpruned"]["value"]
        line["bf16_over_fp32_note"] = ("the BF16 precision form (pruned, FP64 ranking) over the plain FP32 "
                                       "form without pruning; over this line's pruned FP32 value: %.3f"
                                       % (f["bf16_tc"]["value"] / value))
        u = f["fp32_unpruned"]
        line["roofline"]["unpruned"] = {
            "kernel": "csx::screen_q_kernel<true>", "kernel_ms_per_launch": u["screen_kernel_ms"],
            "algorithmic_ops_per_candidate": full_synth_ops(tail),
            "issue_slots": issue_slots(args.lam / (u["screen_kernel_ms"] * 1e-3) * full_synth_ops(tail) / 1e12,
                                       clocks)}
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, args.cpu_seconds)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
