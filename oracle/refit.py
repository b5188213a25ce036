"""FP64 CPU restatement of the surrogate refit (brain/evolve.py:211-268).

TEST INFRASTRUCTURE ONLY: tests/ and bench.py's CPU leg use it as the checker
for the GPU refit (codec_arena_gb300.surrogate); the product never imports it.

`features` follows brain/evolve.py:211-220 ([1 | genes | g_i g_j for j <= i <
16], i outer), `refit_solve` follows :250-268 (normal equations in FP64, then
`np.linalg.solve`), and `refit_cholesky` solves the same system by an FP64
Cholesky factorisation, the form the GPU solve uses. Both are pinned against
outputs of the reference's own refit_surrogate in tests/golden/evolve_golden.json.
With full=True (or 465 coefficients) the quadratic block covers every gene:
the full surface, which has no reference code (docs/RESEARCH_V05C.md:99-102
queues it); its features extend the same pattern.
"""
from __future__ import annotations

import numpy as np


FULL_NF = 465


def _quad_genes(ng: int, full: bool) -> int:
    return ng if full else 16


def features(genes, full: bool = False) -> np.ndarray:
    """(n, ng) genes -> (n, 1 + ng + 136) FP64 features; full: (n, 1 + ng +
    ng(ng+1)/2)."""
    g = np.atleast_2d(np.asarray(genes, dtype=np.float64))
    n = g.shape[0]
    qg = _quad_genes(g.shape[1], full)
    quad = [g[:, i] * g[:, j] for i in range(qg) for j in range(i + 1)]
    return np.concatenate([np.ones((n, 1)), g, np.stack(quad, axis=1)], axis=1)


def normal_equations(genes, fit, full: bool = False):
    X = features(genes, full)
    y = np.asarray(fit, dtype=np.float64)
    return X.T @ X, X.T @ y


def refit_solve(genes, fit, prior, alpha: float) -> np.ndarray:
    """brain/evolve.py:259-265: solve(XᵀX + αI, Xᵀy + α w₀)."""
    XtX, Xty = normal_equations(genes, fit, len(prior) == FULL_NF)
    w0 = np.asarray(prior, dtype=np.float64)
    return np.linalg.solve(XtX + alpha * np.eye(XtX.shape[0]), Xty + alpha * w0)


def cholesky_solve(A, b) -> np.ndarray:
    L = np.linalg.cholesky(A)
    z = np.linalg.solve(L, b)  # L is lower triangular; a general solve is exact enough here
    return np.linalg.solve(L.T, z)


def refit_cholesky(genes, fit, prior, alpha: float) -> np.ndarray:
    XtX, Xty = normal_equations(genes, fit, len(prior) == FULL_NF)
    w0 = np.asarray(prior, dtype=np.float64)
    return cholesky_solve(XtX + alpha * np.eye(XtX.shape[0]), Xty + alpha * w0)


def score(genes, coef) -> np.ndarray:
    return features(genes, len(coef) == FULL_NF) @ np.asarray(coef, dtype=np.float64)


def grad_genes(genes, coef) -> np.ndarray:
    """Analytic d score / d genes in FP64 (n, ng)."""
    g = np.atleast_2d(np.asarray(genes, dtype=np.float64))
    c = np.asarray(coef, dtype=np.float64)
    ng = g.shape[1]
    d = np.tile(c[1:1 + ng], (g.shape[0], 1))
    q = 1 + ng
    for i in range(_quad_genes(ng, len(c) == FULL_NF)):
        for j in range(i + 1):
            d[:, i] += c[q] * g[:, j]
            d[:, j] += c[q] * g[:, i]
            q += 1
    return d
