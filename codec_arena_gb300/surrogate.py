"""The quadratic surrogate as a differentiable torch function, and the GPU
ridge refit (include/csx_surrogate.h).

`score(genes, coef)` is a ``torch.autograd.Function`` whose backward runs the
hand-written kernels: d score / d genes (for gradient-guided mutation) and
d loss / d coefficients (FP64 accumulation). `refit` replaces
brain/evolve.py:250-268 (`refit_surrogate`): it forms the normal equations
ΦᵀΦ and Φᵀy in FP64 on the GPU and solves (ΦᵀΦ + αI) w = Φᵀy + α w₀ by an
FP64 Cholesky factorisation on one CTA. `ridge_grad` is the ridge loss
gradient 2Φᵀ(Φw − y) + 2α(w − w₀) from the backward kernel, which vanishes
at the solution.

Coefficients use the compact layout of brain/evolve.py:211-220: nf = 1 + ng +
136 (153 for 16 genes, 166 for 29), or the full surface's nf = 465 (all 29
genes quadratic: the quad-block extension docs/RESEARCH_V05C.md:99-102
queues; its FP32 forward is the screen's csx_score_full order). Every tensor
must live on a CUDA device; there is no CPU path.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import _lib
from ._lib import SG_BF16, SG_FP32, SG_FP64, check, lib

NQUAD = 136
FULL_NF = _lib.FULL_NF  # 465


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _genes(genes: torch.Tensor) -> torch.Tensor:
    if not genes.is_cuda or genes.dtype != torch.float32 or genes.dim() != 2:
        raise TypeError("genes must be a 2-D float32 CUDA tensor")
    if genes.stride(1) != 1:
        genes = genes.contiguous()
    return genes


def _ng(nf: int) -> int:
    if nf == FULL_NF:
        return 29
    ng = nf - 1 - NQUAD
    if not 16 <= ng <= 29:
        raise ValueError(f"nf={nf}: the compact layouts have 153..166 or 465 coefficients")
    return ng


def workspace(device, nf: int = 166) -> torch.Tensor:
    return torch.empty(int(lib().csx_sg_workspace_bytes(int(nf))), dtype=torch.uint8, device=device)


class _Score(torch.autograd.Function):
    @staticmethod
    def forward(ctx, genes, coef, precision):
        genes = _genes(genes)
        coef_c = coef.detach().to(torch.float32).contiguous()
        nf = coef_c.numel()
        _ng(nf)
        out = torch.empty(genes.shape[0], dtype=torch.float32, device=genes.device)
        check(lib().csx_sg_forward(coef_c.data_ptr(), nf, genes.data_ptr(), genes.shape[0], genes.stride(0),
                                   precision, out.data_ptr(), _stream(genes.device)), "sg_forward")
        ctx.save_for_backward(genes, coef_c)
        ctx.precision = precision
        ctx.coef_dtype = coef.dtype
        return out

    @staticmethod
    def backward(ctx, gout):
        genes, coef_c = ctx.saved_tensors
        gout = gout.detach().to(torch.float32).contiguous()
        want_g, want_c = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        dgenes = torch.empty_like(genes) if want_g else None
        dcoef = torch.empty(coef_c.numel(), dtype=torch.float64, device=genes.device) if want_c else None
        work = workspace(genes.device, coef_c.numel()) if want_c else None
        check(lib().csx_sg_backward(coef_c.data_ptr(), coef_c.numel(), genes.data_ptr(), genes.shape[0],
                                    genes.stride(0), ctx.precision, gout.data_ptr(), _ptr(dgenes), _ptr(dcoef),
                                    _ptr(work), _stream(genes.device)), "sg_backward")
        return dgenes, (dcoef.to(ctx.coef_dtype) if want_c else None), None


def score(genes: torch.Tensor, coef: torch.Tensor, precision: int = SG_FP32) -> torch.Tensor:
    """Φ(genes)·coef per row, differentiable in genes and coef.

    precision: SG_FP32 (FP32 FMAs) or SG_BF16 (genes and coefficients rounded
    to bf16, FP32 accumulation; the backward uses the same rounded values)."""
    if precision not in (SG_FP32, SG_BF16):
        raise ValueError("precision must be SG_FP32 or SG_BF16 (use score_f64 for FP64)")
    return _Score.apply(genes, coef, precision)


def score_f64(genes: torch.Tensor, coef: torch.Tensor) -> torch.Tensor:
    """FP64 forward (no autograd): Φ(genes)·coef with FP64 coefficients."""
    genes = _genes(genes)
    coef = coef.detach().to(torch.float64).contiguous()
    _ng(coef.numel())
    out = torch.empty(genes.shape[0], dtype=torch.float64, device=genes.device)
    check(lib().csx_sg_forward_f64(coef.data_ptr(), coef.numel(), genes.data_ptr(), genes.shape[0], genes.stride(0),
                                   out.data_ptr(), _stream(genes.device)), "sg_forward_f64")
    return out


def normal_equations(genes: torch.Tensor, fit: Optional[torch.Tensor], nf: int):
    """(ΦᵀΦ, Φᵀy) in FP64 on the GPU (fixed summation order)."""
    genes = _genes(genes)
    _ng(nf)
    dev = genes.device
    gram = torch.empty((nf, nf), dtype=torch.float64, device=dev)
    rhs = torch.empty(nf, dtype=torch.float64, device=dev) if fit is not None else None
    y = fit.detach().to(device=dev, dtype=torch.float64).contiguous() if fit is not None else None
    work = workspace(dev, nf)
    check(lib().csx_sg_normal_equations(nf, genes.data_ptr(), genes.shape[0], genes.stride(0), _ptr(y),
                                        gram.data_ptr(), _ptr(rhs), work.data_ptr(), _stream(dev)),
          "sg_normal_equations")
    return gram, rhs


def ridge_solve(gram: torch.Tensor, rhs: torch.Tensor, alpha: float, prior: Optional[torch.Tensor] = None):
    """w = (G + αI)⁻¹ (rhs + α·prior), FP64 Cholesky on one CTA (the factor in
    shared memory up to 166 coefficients, in a global scratch for 465)."""
    nf = gram.shape[0]
    dev = gram.device
    gram = gram.to(torch.float64).contiguous()
    rhs = rhs.to(torch.float64).contiguous()
    pr = prior.detach().to(device=dev, dtype=torch.float64).contiguous() if prior is not None else None
    w = torch.empty(nf, dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    check(lib().csx_sg_ridge_solve(nf, gram.data_ptr(), rhs.data_ptr(), float(alpha), _ptr(pr), w.data_ptr(),
                                   status.data_ptr(), _stream(dev)), "sg_ridge_solve")
    st = int(status.item())
    if st:
        raise _lib.CsxError(_lib.ERR_BAD_ARGS, f"normal equations not positive definite at pivot {st - 1}")
    return w


def refit(genes: torch.Tensor, fit: torch.Tensor, prior: torch.Tensor, alpha: float = 50.0) -> torch.Tensor:
    """Ridge refit toward the prior (brain/evolve.py:250-268), on the GPU.

    genes: (n, ldg) float32 rows; fit: (n,) targets; prior: (nf,) weights.
    Returns w (nf,) float64."""
    nf = int(prior.numel())
    gram, rhs = normal_equations(genes, fit, nf)
    return ridge_solve(gram, rhs, alpha, prior)


def ridge_grad(genes: torch.Tensor, fit: torch.Tensor, w: torch.Tensor, prior: torch.Tensor,
               alpha: float) -> torch.Tensor:
    """d/dw [ ||Φw − y||² + α||w − w₀||² ] = 2Φᵀ(Φw − y) + 2α(w − w₀), FP64,
    from the FP64 forward and the coefficient backward kernel."""
    genes = _genes(genes)
    dev = genes.device
    w = w.detach().to(device=dev, dtype=torch.float64).contiguous()
    nf = w.numel()
    resid = score_f64(genes, w) - fit.detach().to(device=dev, dtype=torch.float64)
    resid = resid.contiguous()
    g = torch.empty(nf, dtype=torch.float64, device=dev)
    work = workspace(dev, nf)
    check(lib().csx_sg_backward_coef_f64(nf, genes.data_ptr(), genes.shape[0], genes.stride(0), resid.data_ptr(),
                                         g.data_ptr(), work.data_ptr(), _stream(dev)), "sg_backward_coef_f64")
    pr = prior.detach().to(device=dev, dtype=torch.float64)
    return 2.0 * g + 2.0 * alpha * (w - pr)


def ascend(genes: torch.Tensor, coef: torch.Tensor, eta: float, steps: int):
    """Gradient-guided mutation: `steps` projected ascent steps
    g <- clamp01(g + eta·∇score(g)) on a copy of `genes`.
    Returns (new genes, FP32 scores)."""
    out = _genes(genes).clone()
    coef = coef.detach().to(device=out.device, dtype=torch.float32).contiguous()
    nf = coef.numel()
    _ng(nf)
    sc = torch.empty(out.shape[0], dtype=torch.float32, device=out.device)
    check(lib().csx_sg_ascend(coef.data_ptr(), nf, out.data_ptr(), out.shape[0], out.stride(0), float(eta),
                              int(steps), sc.data_ptr(), _stream(out.device)), "sg_ascend")
    return out, sc


__all__ = ["score", "score_f64", "normal_equations", "ridge_solve", "refit", "ridge_grad", "ascend",
           "SG_FP32", "SG_BF16", "SG_FP64"]
