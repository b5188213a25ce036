"""Seeded synthetic inputs for the screen (no dataset is involved).

* ``seeded_elites``: n genomes whose 29 genes are splitmix64 unit() draws from
  one seed, written to 4 decimals (the pop-line text format every elite passes
  through, brain/evolve.py:104-106) and read back as f32; ids 0..n-1, tribe =
  id % 12.
* ``seeded_normal_model``: compact surrogate weights N(0, 1) * scale drawn by
  Box-Muller in f64 on a splitmix64 stream, rounded to f32.
* ``load_compact``: the compact weights of a surrogate text file.

splitmix64 here is the published generator (the same one src/screen.zig:195-213
uses), evaluated with numpy uint64 arithmetic.
"""
from __future__ import annotations

import os

import numpy as np

from .genome import make_genomes

G = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests",
                          "golden")
SURROGATE_161 = os.path.join(GOLDEN_DIR, "surrogate_v3_161.txt")


def splitmix64(seed: int, n: int) -> np.ndarray:
    """First n outputs of splitmix64 seeded with ``seed``."""
    with np.errstate(over="ignore"):
        k = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * G
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        return z ^ (z >> np.uint64(31))


def units(seed: int, n: int) -> np.ndarray:
    """unit() of src/screen.zig:210-213: f32(next() >> 40) * 2^-24."""
    return (splitmix64(seed, n) >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def seeded_elites(n: int = 64, seed: int = 1) -> np.ndarray:
    u = units(seed, n * 29).reshape(n, 29)
    # %.4f of the f32 value, read back as f32 (4-decimal text is never an f32
    # rounding midpoint, so float() then float32 rounds correctly)
    g = np.array([[np.float32(float(f"{float(x):.4f}")) for x in row] for row in u], dtype=np.float32)
    ids = np.arange(n, dtype=np.uint64)
    return make_genomes(g, ids=ids, tribes=(ids % 12).astype(np.uint32))


def seeded_normal_model(seed: int = 2, n: int = 153, scale: float = 0.1) -> np.ndarray:
    """Compact weights, N(0,1)*scale by Box-Muller (f64) on splitmix64(seed)."""
    x = splitmix64(seed, 2 * n)
    u = (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)  # [0, 1)
    u1, u2 = u[0::2], u[1::2]
    z = np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)
    return (z * scale).astype(np.float32)


def load_compact(path: str) -> np.ndarray:
    with open(path) as f:
        toks = f.read().split()
    n = int(toks[0])
    return np.array([np.float32(t) for t in toks[1:1 + n]], dtype=np.float32)


def surrogate_161() -> np.ndarray:
    """The reference's committed v3 surrogate (161 coefficients), from the fixture."""
    return load_compact(SURROGATE_161)


def refit_table(n: int = 400_000, seed: int = 5, ng: int = 16, noise: float = 0.5):
    """Synthetic refit table: n rows of `ng` genes uniform in [0, 1] (f32),
    targets = a seeded ground-truth quadratic (N(0, 1) coefficients, FP64) plus
    Student-t(3) noise of scale `noise`. Returns (genes, fit, w_true)."""
    rng = np.random.default_rng(seed)
    genes = rng.random((n, ng), dtype=np.float32)
    nf = 1 + ng + 136
    w_true = rng.normal(0.0, 1.0, nf)
    g = genes.astype(np.float64)
    ii, jj = np.tril_indices(16)
    fit = w_true[0] + g @ w_true[1:1 + ng] + (g[:, ii] * g[:, jj]) @ w_true[1 + ng:]
    fit = fit + noise * rng.standard_t(3, n)
    return genes, fit, w_true


def refit_table_full(n: int = 400_000, seed: int = 6, noise: float = 0.5):
    """Synthetic refit table for the full surface: n rows of 29 genes uniform
    in [0, 1] (f32), targets = a seeded quadratic over all 29 genes (465
    N(0, 1) coefficients, FP64) plus Student-t(3) noise of scale `noise`.
    Returns (genes, fit, w_true)."""
    rng = np.random.default_rng(seed)
    genes = rng.random((n, 29), dtype=np.float32)
    w_true = rng.normal(0.0, 1.0, 465)
    g = genes.astype(np.float64)
    ii, jj = np.tril_indices(29)
    fit = w_true[0] + g @ w_true[1:30]
    for a in range(0, n, 50_000):  # the 435 products in row blocks (bounded host memory)
        b = min(n, a + 50_000)
        fit[a:b] += (g[a:b, ii] * g[a:b, jj]) @ w_true[30:]
    fit = fit + noise * rng.standard_t(3, n)
    return genes, fit, w_true


def seeded_islands(n: int = 20, seed: int = 4, lam_lo: float = 1e8, lam_hi: float = 2.65e9,
                   ne_lo: int = 16, ne_hi: int = 256, keeps=(32, 128, 256), threads: int = 4):
    """Batched-islands workload: n islands with log-uniform budgets in
    [lam_lo, lam_hi], elite pools of ne_lo..ne_hi seeded genomes, each island
    with its own seeded N(0, 0.1) 153-coefficient surface and a top-K from
    `keeps`. Returns a list of dicts (lambda, keep, seed, threads, elites,
    weights)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        lam = int(round(float(np.exp(rng.uniform(np.log(lam_lo), np.log(lam_hi))))))
        ne = int(rng.integers(ne_lo, ne_hi + 1))
        keep = int(keeps[int(rng.integers(0, len(keeps)))])
        out.append({"lambda": lam, "keep": keep, "seed": 100 + i, "threads": threads,
                    "elites": seeded_elites(ne, seed=1000 + i),
                    "weights": seeded_normal_model(seed=2000 + i)})
    return out
