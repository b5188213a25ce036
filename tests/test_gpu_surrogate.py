"""The differentiable surrogate and the GPU ridge refit against the FP64 oracle
(oracle/refit.py), finite differences and FP64 torch autograd.

Tolerances: FP32 forward within 1e-5 of the FP64 score relative to the sum of
absolute terms; gene gradients likewise; coefficient gradients, normal
equations and the refit (FP64 throughout) within 1e-9 relative.
"""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(ROOT, "oracle"))


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(csx):
    from conftest import has_gpu

    if not has_gpu():
        pytest.skip("no CUDA device")


def _case(n, ng, seed):
    rng = np.random.default_rng(seed)
    genes = rng.random((n, ng), dtype=np.float32)
    coef = rng.normal(0, 1, 1 + ng + 136).astype(np.float32)
    return genes, coef


def _abs_scale(genes, coef):
    import refit

    return np.abs(refit.features(genes)) @ np.abs(coef.astype(np.float64))


def _bf16(x):
    import torch

    return torch.from_numpy(np.asarray(x, dtype=np.float32)).to(torch.bfloat16).to(torch.float32).numpy()


@pytest.mark.parametrize("ng", [16, 22, 24, 27, 28, 29])
def test_forward_fp32_vs_fp64_oracle(ng):
    import refit
    import torch

    from codec_arena_gb300 import surrogate

    genes, coef = _case(5000, ng, ng)
    got = surrogate.score(torch.from_numpy(genes).cuda(), torch.from_numpy(coef).cuda()).cpu().numpy()
    want = refit.score(genes, coef)
    assert np.all(np.abs(got - want) <= 1e-5 * _abs_scale(genes, coef))


def test_forward_bf16_and_fp64():
    import refit
    import torch

    from codec_arena_gb300 import surrogate

    genes, coef = _case(4000, 29, 1)
    d = torch.from_numpy(genes).cuda()
    got = surrogate.score(d, torch.from_numpy(coef).cuda(), surrogate.SG_BF16).cpu().numpy()
    want = refit.score(_bf16(genes), _bf16(coef))
    assert np.all(np.abs(got - want) <= 1e-5 * _abs_scale(_bf16(genes), _bf16(coef)))
    # the bf16 form against the exact score: its error is the input rounding
    err = np.abs(got - refit.score(genes, coef)) / _abs_scale(genes, coef)
    assert err.max() < 2 ** -7
    got64 = surrogate.score_f64(d, torch.from_numpy(coef.astype(np.float64)).cuda()).cpu().numpy()
    np.testing.assert_allclose(got64, refit.score(genes, coef), rtol=1e-13, atol=1e-13)


def test_ldg_stride_and_empty():
    import refit
    import torch

    from codec_arena_gb300 import surrogate

    genes, coef = _case(777, 29, 3)
    wide = np.zeros((777, 40), np.float32)
    wide[:, :16] = genes[:, :16]
    wide[:, 16:] = 0.75  # beyond ng: never read
    c16 = np.concatenate([coef[:17], coef[30:]])  # v1 layout: 153
    got = surrogate.score(torch.from_numpy(wide).cuda(), torch.from_numpy(c16).cuda()).cpu().numpy()
    want = refit.score(genes[:, :16], c16)
    assert np.all(np.abs(got - want) <= 1e-5 * _abs_scale(genes[:, :16], c16))
    e = surrogate.score(torch.zeros((0, 29), device="cuda"), torch.from_numpy(coef).cuda())
    assert e.shape == (0,)


def test_gene_gradient_vs_oracle_and_torch_f64():
    import refit
    import torch

    from codec_arena_gb300 import surrogate

    genes, coef = _case(3000, 29, 4)
    g = torch.from_numpy(genes).cuda().requires_grad_(True)
    c = torch.from_numpy(coef).cuda()
    gout = torch.from_numpy(np.random.default_rng(5).normal(size=3000).astype(np.float32)).cuda()
    (surrogate.score(g, c) * gout).sum().backward()
    got = g.grad.cpu().numpy()
    want = refit.grad_genes(genes, coef) * gout.cpu().numpy()[:, None].astype(np.float64)
    scale = np.abs(coef).sum() * np.abs(gout.cpu().numpy())[:, None]
    assert np.all(np.abs(got - want) <= 1e-5 * scale)
    # FP64 torch autograd through the features
    g64 = torch.from_numpy(genes.astype(np.float64)).cuda().requires_grad_(True)
    ii, jj = np.tril_indices(16)
    phi = torch.cat([torch.ones(3000, 1, dtype=torch.float64, device="cuda"), g64, g64[:, ii] * g64[:, jj]], 1)
    (phi @ torch.from_numpy(coef.astype(np.float64)).cuda() * gout.double()).sum().backward()
    assert np.all(np.abs(got - g64.grad.cpu().numpy()) <= 1e-5 * scale)


def _fd_check(genes, coef, precision, h, scale_coef):
    """Central differences of the forward in `precision` against the backward.
    The surrogate is quadratic, so a central difference has no truncation
    error; what remains is the forward's FP32 rounding (bounded by 1e-5 of the
    absolute-term sum) divided by h."""
    import torch

    from codec_arena_gb300 import surrogate

    c = torch.from_numpy(coef).cuda()
    g = torch.from_numpy(genes).cuda().requires_grad_(True)
    surrogate.score(g, c, precision).sum().backward()
    grad = g.grad.cpu().numpy()
    for k in range(genes.shape[1]):
        gp, gm = genes.copy(), genes.copy()
        gp[:, k] += h
        gm[:, k] -= h
        fp = surrogate.score(torch.from_numpy(gp).cuda(), c, precision).double().cpu().numpy()
        fm = surrogate.score(torch.from_numpy(gm).cuda(), c, precision).double().cpu().numpy()
        fd = (fp - fm) / (2 * h)
        tol = 1e-5 * np.maximum(_abs_scale(gp, scale_coef), _abs_scale(gm, scale_coef)) / h
        assert np.all(np.abs(fd - grad[:, k]) <= tol + 1e-5 * np.abs(scale_coef).sum()), k


def test_gene_gradient_finite_differences_fp32():
    from codec_arena_gb300 import surrogate

    genes, coef = _case(512, 29, 6)
    _fd_check(genes, coef, surrogate.SG_FP32, 0.25, coef)


def test_gene_gradient_finite_differences_bf16():
    """Genes on the grid k/256 and steps of 1/16 stay exact in bf16, so central
    differences of the bf16 forward see the same rounded inputs as its
    gradient."""
    from codec_arena_gb300 import surrogate

    rng = np.random.default_rng(7)
    genes = (rng.integers(16, 240, size=(512, 29)) / 256.0).astype(np.float32)
    coef = rng.normal(0, 1, 166).astype(np.float32)
    _fd_check(genes, coef, surrogate.SG_BF16, 1.0 / 16, _bf16(coef))


def test_coefficient_gradient_fp64():
    import refit
    import torch

    from codec_arena_gb300 import surrogate

    genes, coef = _case(20000, 29, 8)
    gout = np.random.default_rng(9).normal(size=20000).astype(np.float32)
    c = torch.from_numpy(coef).cuda().requires_grad_(True)
    out = surrogate.score(torch.from_numpy(genes).cuda(), c)
    out.backward(torch.from_numpy(gout).cuda())
    want = refit.features(genes).T @ gout.astype(np.float64)
    scale = np.abs(refit.features(genes)).T @ np.abs(gout.astype(np.float64))
    assert np.all(np.abs(c.grad.double().cpu().numpy() - want) <= 1e-6 * scale)  # the f32 cast of the output
    # the FP64 entry point directly
    d = torch.empty(166, dtype=torch.float64, device="cuda")
    w = surrogate.workspace("cuda")
    g_d = torch.from_numpy(genes).cuda()
    go = torch.from_numpy(gout.astype(np.float64)).cuda()
    from codec_arena_gb300._lib import check, lib

    check(lib().csx_sg_backward_coef_f64(166, g_d.data_ptr(), 20000, 29, go.data_ptr(), d.data_ptr(), w.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream))
    assert np.all(np.abs(d.cpu().numpy() - want) <= 1e-12 * scale)


@pytest.mark.parametrize("ng", [16, 29])
def test_normal_equations_vs_oracle(ng):
    import refit
    import torch

    from codec_arena_gb300 import surrogate

    genes, _ = _case(50000, ng, 10 + ng)
    fit = np.random.default_rng(11).normal(size=50000)
    G, r = surrogate.normal_equations(torch.from_numpy(genes).cuda(), torch.from_numpy(fit).cuda(), 1 + ng + 136)
    Gw, rw = refit.normal_equations(genes, fit)
    np.testing.assert_allclose(G.cpu().numpy(), Gw, rtol=1e-12)
    X = np.abs(refit.features(genes))
    assert np.all(np.abs(r.cpu().numpy() - rw) <= 1e-12 * (X.T @ np.abs(fit)))
    G2, _ = surrogate.normal_equations(torch.from_numpy(genes).cuda(), torch.from_numpy(fit).cuda(), 1 + ng + 136)
    assert torch.equal(G, G2)  # fixed summation order


def test_refit_matches_reference_golden():
    """brain/evolve.py's own refit_surrogate output (400 rows, alpha 50), as
    written by save_weights ("%.8e")."""
    import json

    import torch

    from codec_arena_gb300 import surrogate

    with open(os.path.join(ROOT, "tests", "golden", "evolve_golden.json")) as f:
        r = json.load(f)["refit"]
    genes = torch.tensor(r["rows_genes"], dtype=torch.float64)
    # the reference computes features from f64 genes; these rows are f32-exact only after rounding
    g32 = genes.float()
    f64 = dict(dtype=torch.float64, device="cuda")
    w = surrogate.refit(g32.cuda(), torch.tensor(r["rows_fit"], **f64), torch.tensor(r["prior"], **f64), r["alpha"])
    import refit

    want = refit.refit_cholesky(g32.numpy(), r["rows_fit"], r["prior"], r["alpha"])
    np.testing.assert_allclose(w.cpu().numpy(), want, rtol=1e-9, atol=1e-12)
    # against the golden file (f64 genes, 9 significant digits): the f32 rounding
    # of the genes moves the solution by 2.5e-8 at most
    np.testing.assert_allclose(w.cpu().numpy(), r["weights"], rtol=0, atol=1e-7)


def test_refit_400k_student_t_vs_fp64_cholesky():
    import refit
    import torch

    from codec_arena_gb300 import surrogate, workloads as wl

    genes, fit, w_true = wl.refit_table()
    prior = np.zeros(153)
    d_g = torch.from_numpy(genes).cuda()
    d_y = torch.from_numpy(fit).cuda()
    w = surrogate.refit(d_g, d_y, torch.from_numpy(prior).cuda(), alpha=1e-2)
    want = refit.refit_cholesky(genes, fit, prior, 1e-2)
    err = np.abs(w.cpu().numpy() - want).max() / np.abs(want).max()
    assert err < 1e-9, err
    # the ridge-loss gradient from the backward kernel vanishes at the solution
    gr = surrogate.ridge_grad(d_g, d_y, w, torch.from_numpy(prior).cuda(), 1e-2).cpu().numpy()
    X = refit.features(genes)
    scale = 2 * (np.abs(X).T @ (np.abs(X) @ np.abs(want) + np.abs(fit)))
    assert np.abs(gr).max() <= 1e-10 * scale.max()
    # and equals the FP64 oracle gradient at another point
    w1 = want + np.random.default_rng(1).normal(0, 0.1, 153)
    gr1 = surrogate.ridge_grad(d_g, d_y, torch.from_numpy(w1).cuda(), torch.from_numpy(prior).cuda(), 1e-2)
    want1 = 2 * X.T @ (X @ w1 - fit) + 2e-2 * (w1 - prior)
    np.testing.assert_allclose(gr1.cpu().numpy(), want1, rtol=1e-9, atol=1e-9 * np.abs(want1).max())


def test_ridge_solve_reports_indefinite():
    import torch

    from codec_arena_gb300 import _lib, surrogate

    G = torch.zeros((153, 153), dtype=torch.float64, device="cuda")
    G[5, 5] = -1.0
    with pytest.raises(_lib.CsxError, match="pivot"):
        surrogate.ridge_solve(G, torch.zeros(153, dtype=torch.float64, device="cuda"), 0.5)


def test_gradient_ascent_mutation():
    import torch

    from codec_arena_gb300 import surrogate

    genes, coef = _case(4096, 29, 12)
    c = torch.from_numpy(coef).cuda()
    d = torch.from_numpy(genes).cuda()
    s0 = surrogate.score(d, c)
    L = np.abs(coef[30:]).sum() * 2  # a bound on the Hessian's norm
    eta = 0.5 / L
    g1, s1 = surrogate.ascend(d, c, eta, 10)
    assert torch.equal(d, torch.from_numpy(genes).cuda())  # input untouched
    assert g1.min() >= 0 and g1.max() <= 1
    assert torch.all(s1 >= s0 - 1e-4 * s0.abs().max())
    assert float((s1 - s0).mean()) > 0
    # the same steps in FP64 torch
    g = torch.from_numpy(genes.astype(np.float64)).cuda()
    c64 = c.double()
    ii, jj = np.tril_indices(16)
    for _ in range(10):
        g.requires_grad_(True)
        phi = torch.cat([torch.ones(4096, 1, dtype=torch.float64, device="cuda"), g, g[:, ii] * g[:, jj]], 1)
        (phi @ c64).sum().backward()
        g = (g + eta * g.grad).clamp(0, 1).detach()
    assert (g1.double() - g).abs().max() < 1e-4


def test_bad_arguments():
    import torch

    from codec_arena_gb300 import _lib, surrogate

    with pytest.raises(ValueError):
        surrogate.score(torch.zeros((4, 29), device="cuda"), torch.zeros(150, device="cuda"))
    with pytest.raises(TypeError):
        surrogate.score(torch.zeros((4, 29)), torch.zeros(166))
    with pytest.raises(_lib.CsxError):
        surrogate.score(torch.zeros((4, 20), device="cuda"), torch.zeros(166, device="cuda"))


# ---- the full surface (465 coefficients: all 29 genes quadratic) ---------------------

def _full_case(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    genes = rng.random((n, 29), dtype=np.float32)
    coef = (rng.normal(0, 1, 465) * scale).astype(np.float32)
    return genes, coef


def test_full_forward_is_the_screen_score():
    """The FP32 forward of the full layout evaluates csx_score_full's FMA
    order: bit-equal to the screen's score of the same genes, and within the
    FP32 bound of the FP64 oracle."""
    import refit
    import torch

    from codec_arena_gb300 import screen, surrogate

    genes, coef = _full_case(4000, 1)
    d_g = torch.from_numpy(genes).cuda()
    got = surrogate.score(d_g, torch.from_numpy(coef).cuda()).cpu().numpy()
    scr = screen.score_genes(screen.ModelFull.from_compact(coef), d_g).cpu().numpy()
    np.testing.assert_array_equal(got.view(np.uint32), scr.view(np.uint32))
    X = np.abs(refit.features(genes, full=True))
    assert np.all(np.abs(got - refit.score(genes, coef)) <= 1e-5 * (X @ np.abs(coef.astype(np.float64))))
    g64 = surrogate.score_f64(d_g, torch.from_numpy(coef.astype(np.float64)).cuda()).cpu().numpy()
    np.testing.assert_allclose(g64, refit.score(genes, coef), rtol=1e-12, atol=1e-12)


def test_full_gene_gradient_and_coefficient_gradient():
    import refit
    import torch

    from codec_arena_gb300 import surrogate

    genes, coef = _full_case(3000, 2)
    g = torch.from_numpy(genes).cuda().requires_grad_(True)
    c = torch.from_numpy(coef.astype(np.float64)).cuda().requires_grad_(True)
    s = surrogate.score(g, c)
    gout = torch.from_numpy(np.random.default_rng(3).normal(size=3000).astype(np.float32)).cuda()
    (s * gout).sum().backward()
    want_g = refit.grad_genes(genes, coef) * gout.cpu().numpy()[:, None].astype(np.float64)
    scale = np.abs(refit.grad_genes(genes, np.abs(coef))).max()
    assert np.abs(g.grad.cpu().numpy() - want_g).max() <= 1e-5 * scale * np.abs(gout.cpu().numpy()).max()
    want_c = refit.features(genes, full=True).T @ gout.cpu().numpy().astype(np.float64)
    np.testing.assert_allclose(c.grad.cpu().numpy(), want_c, rtol=1e-9, atol=1e-9 * np.abs(want_c).max())


def test_full_normal_equations_and_refit():
    """465 features: ΦᵀΦ spans 6903 4x4 blocks over seven CTA columns; the
    Cholesky factor (108k entries) lives in a global scratch."""
    import refit
    import torch

    from codec_arena_gb300 import surrogate

    rng = np.random.default_rng(7)
    n = 60000
    genes = rng.random((n, 29), dtype=np.float32)
    w_true = rng.normal(0, 1, 465)
    fit = refit.features(genes, full=True) @ w_true + rng.standard_t(3, n) * 0.5
    d_g, d_y = torch.from_numpy(genes).cuda(), torch.from_numpy(fit).cuda()
    G, r = surrogate.normal_equations(d_g, d_y, 465)
    Gw, rw = refit.normal_equations(genes, fit, full=True)
    np.testing.assert_allclose(G.cpu().numpy(), Gw, rtol=1e-12)
    X = np.abs(refit.features(genes, full=True))
    assert np.all(np.abs(r.cpu().numpy() - rw) <= 1e-12 * (X.T @ np.abs(fit)))
    G2, _ = surrogate.normal_equations(d_g, d_y, 465)
    assert torch.equal(G, G2)
    prior = rng.normal(0, 0.1, 465)
    w = surrogate.refit(d_g, d_y, torch.from_numpy(prior).cuda(), alpha=1e-2).cpu().numpy()
    want = refit.refit_cholesky(genes, fit, prior, 1e-2)
    assert np.abs(w - want).max() <= 1e-8 * np.abs(want).max()
    assert np.abs(w - w_true).max() < 0.5  # the fit recovers the surface


def test_full_ascent_raises_the_score():
    import torch

    from codec_arena_gb300 import surrogate

    genes, coef = _full_case(2000, 5, 0.2)
    d_c = torch.from_numpy(coef).cuda()
    d_g = torch.from_numpy(genes).cuda()
    before = surrogate.score(d_g, d_c)
    new, after = surrogate.ascend(d_g, d_c, 1e-3, 10)
    assert (after >= before - 1e-4).float().mean().item() > 0.99
    assert after.mean().item() > before.mean().item()
    assert float(new.min()) >= 0.0 and float(new.max()) <= 1.0
    np.testing.assert_array_equal(after.cpu().numpy(), surrogate.score(new, d_c).detach().cpu().numpy())
