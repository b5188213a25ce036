"""The precision form of the surrogate score: the quadratic block on the
tensor cores (tcgen05, FP32 accumulation) with genes in BF16, or in FP16 with
the per-gene map x' = 2g - 1 onto [-1, 1]; constant and linear terms in FP32.
The reference scores in FP32 only (src/screen.zig:97-112); this form exists to
trade score precision for tensor-core throughput, with its error measured
against FP64.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import TC_BF16, TC_FP16, check, lib
from .screen import Model

FORMS = {"bf16": TC_BF16, "fp16": TC_FP16}


def tc_score(model: Model, genes, form: str = "bf16"):
    """Score rows of a (n, >=29) float32 CUDA tensor; returns float32 scores."""
    import torch

    if not genes.is_cuda or genes.dtype != torch.float32 or genes.dim() != 2 or genes.stride(1) != 1:
        raise TypeError("genes must be a contiguous-row 2-D float32 CUDA tensor")
    n = genes.shape[0]
    out = torch.empty(n, dtype=torch.float32, device=genes.device)
    err = torch.zeros(1, dtype=torch.int32, device=genes.device)
    check(lib().csx_tc_score(ctypes.byref(model.c), FORMS[form], genes.data_ptr(), n, genes.stride(0),
                             out.data_ptr(), err.data_ptr(), torch.cuda.current_stream(genes.device).cuda_stream),
          "tc_score")
    if int(err.item()):
        raise _lib.CsxError(_lib.ERR_DEVICE_STATE, f"tensor-core wait gave up (bits {int(err.item())})")
    return out


__all__ = ["tc_score", "FORMS"]
