"""The screen funnel's Python API, mirroring src/screen.zig.

``Model.from_compact`` / ``load_model`` / ``Cfg`` / ``run`` keep the names and
argument meaning of the Zig module; ``screen`` returns the survivors as a
numpy record array instead of writing files, and ``screen_device`` runs on
torch-owned device memory and the current torch CUDA stream.

Everything computes on the GPU through libcsx_screen.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Optional, Tuple

import numpy as np

from . import _lib
from ._lib import GENOME_DTYPE, NTOT, SURVIVOR_DTYPE, CsxError, check, lib

VALID_N = (153, 159, 161, 164, 165, 166)


class Model:
    """Model (src/screen.zig:23-27): w0, w_lin[29], w_quad[16*16] lower-triangular."""

    def __init__(self, c: _lib.CsxModel):
        self._c = c

    @classmethod
    def from_compact(cls, w) -> "Model":
        """Model.fromCompact, src/screen.zig:36-95."""
        w = np.ascontiguousarray(w, dtype=np.float32)
        c = _lib.CsxModel()
        check(lib().csx_model_from_compact(w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                           int(w.shape[0]), ctypes.byref(c)), "fromCompact")
        return cls(c)

    @property
    def w0(self) -> float:
        return float(self._c.w0)

    @property
    def w_lin(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._c.w_lin).copy()

    @property
    def w_quad(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._c.w_quad).copy()

    @property
    def c(self) -> _lib.CsxModel:
        return self._c


class ModelFull:
    """The full quadratic surface over all 29 genes (465 compact floats):
    the quad-block extension docs/RESEARCH_V05C.md:99-102 queues, which the
    reference's code does not have. Its score order is csx_screen.h's."""

    NF = _lib.FULL_NF

    def __init__(self, c: _lib.CsxModelFull):
        self._c = c

    @classmethod
    def from_compact(cls, w) -> "ModelFull":
        w = np.ascontiguousarray(w, dtype=np.float32)
        c = _lib.CsxModelFull()
        check(lib().csx_model_full_from_compact(w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                int(w.shape[0]), ctypes.byref(c)), "full fromCompact")
        return cls(c)

    @property
    def w0(self) -> float:
        return float(self._c.w0)

    @property
    def w_lin(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._c.w_lin).copy()

    @property
    def w_quad(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._c.w_quad).copy()

    @property
    def c(self) -> _lib.CsxModelFull:
        return self._c


def parse_model_text(text: str) -> np.ndarray:
    """loadModel's text body, src/screen.zig:118-126: returns the compact weights."""
    b = text.encode()
    w = (ctypes.c_float * 166)()
    n = ctypes.c_int(0)
    check(lib().csx_model_parse(b, len(b), w, 166, ctypes.byref(n)), "loadModel")
    return np.array(w[: n.value], dtype=np.float32)


def load_model(path: str) -> Model:
    """loadModel, src/screen.zig:115-127 (1 MiB file limit as in the reference)."""
    with open(path, "rb") as f:
        data = f.read((1 << 20) + 1)
    if len(data) > (1 << 20):
        raise CsxError(_lib.ERR_IO, f"{path}: larger than 1 MiB")
    return Model.from_compact(parse_model_text(data.decode()))


@dataclass
class Cfg:
    """Cfg, src/screen.zig:129-137. ``threads`` is the RNG stream count T."""

    lambda_: int
    keep: int
    seed: int
    threads: int = 4
    sigma: float = 0.12
    jump_p: float = 0.02
    imm_p: float = 0.01
    flags: int = 0

    def c(self) -> _lib.CsxCfg:
        return _lib.CsxCfg(int(self.lambda_), int(self.keep), int(self.seed), int(self.threads),
                           float(self.sigma), float(self.jump_p), float(self.imm_p), int(self.flags))


def _elites_array(elites) -> np.ndarray:
    e = np.ascontiguousarray(elites)
    if e.dtype != GENOME_DTYPE:
        raise TypeError("elites must be a GENOME_DTYPE array (see genome.make_genomes)")
    return e


def screen(cfg: Cfg, model: Model, elites, streams: Optional[Tuple[int, int]] = None,
           items: Optional[Tuple[int, int]] = None) -> Tuple[np.ndarray, int]:
    """run() without the file output: (survivors sorted by score desc, screened).

    streams=(a, b) screens only RNG streams a..b-1 of the generation (one
    rank's share when a generation is sharded by stream; an empty range gives
    no survivors and screens nothing). items=(r, W) screens share r of W of
    the generation's work items (any number of ranks, even more than
    streams). Merge the ranks' survivors with parallel.merge_survivors. A
    ModelFull scores the candidates on the full 29-gene quadratic surface
    instead (stream ranges only)."""
    e = _elites_array(elites)
    keep_n = min(int(cfg.keep), int(cfg.lambda_))
    out = np.zeros(max(keep_n, 1), dtype=SURVIVOR_DTYPE)
    n_out = ctypes.c_uint64(0)
    screened = ctypes.c_uint64(0)
    c = cfg.c()
    if streams is not None and int(streams[0]) == int(streams[1]):
        return out[:0], 0  # a rank with no stream of its own (more ranks than streams)
    if items is not None:
        if isinstance(model, ModelFull) or streams is not None:
            raise ValueError("items= shards the reference surface's whole generation")
        check(lib().csx_screen_items(ctypes.byref(c), ctypes.byref(model.c), e.ctypes.data, int(e.shape[0]),
                                     int(items[0]), int(items[1]), out.ctypes.data, keep_n, ctypes.byref(n_out),
                                     ctypes.byref(screened)), "screen_items")
        return out[: n_out.value], int(screened.value)
    if isinstance(model, ModelFull) and streams is None:
        check(lib().csx_screen_full(ctypes.byref(c), ctypes.byref(model.c), e.ctypes.data, int(e.shape[0]),
                                    out.ctypes.data, keep_n, ctypes.byref(n_out), ctypes.byref(screened)),
              "screen_full")
    elif isinstance(model, ModelFull):
        check(lib().csx_screen_full_range(ctypes.byref(c), ctypes.byref(model.c), e.ctypes.data, int(e.shape[0]),
                                          int(streams[0]), int(streams[1]), out.ctypes.data, keep_n,
                                          ctypes.byref(n_out), ctypes.byref(screened)), "screen_full_range")
    elif streams is None:
        check(lib().csx_screen(ctypes.byref(c), ctypes.byref(model.c), e.ctypes.data, int(e.shape[0]),
                               out.ctypes.data, keep_n, ctypes.byref(n_out), ctypes.byref(screened)),
              "screen")
    else:
        check(lib().csx_screen_range(ctypes.byref(c), ctypes.byref(model.c), e.ctypes.data, int(e.shape[0]),
                                     int(streams[0]), int(streams[1]), out.ctypes.data, keep_n,
                                     ctypes.byref(n_out), ctypes.byref(screened)), "screen_range")
    return out[: n_out.value], int(screened.value)


def score_genes(model: Model, genes):
    """Model.score (src/screen.zig:97-112) of the rows of a (n, >=29) float32
    CUDA tensor, in the reference's f32 order, on the GPU (a ModelFull: the
    full surface's score in its FMA order)."""
    import torch

    if not genes.is_cuda or genes.dtype != torch.float32 or genes.dim() != 2 or genes.stride(1) != 1:
        raise TypeError("genes must be a 2-D float32 CUDA tensor with contiguous rows")
    out = torch.empty(genes.shape[0], dtype=torch.float32, device=genes.device)
    fn = lib().csx_score_full if isinstance(model, ModelFull) else lib().csx_score
    check(fn(ctypes.byref(model.c), genes.data_ptr(), genes.shape[0], genes.stride(0), out.data_ptr(),
             torch.cuda.current_stream(genes.device).cuda_stream), "score")
    return out


def format_survivor(rec, flags: int = 0) -> str:
    """One promoted line (src/screen.zig:327-336 with FLAG_OUTPUT_29, else v6)."""
    buf = ctypes.create_string_buffer(1024)
    arr = np.ascontiguousarray(np.asarray(rec, dtype=SURVIVOR_DTYPE).reshape(1))
    n = check(lib().csx_survivor_format_line(arr.ctypes.data, int(flags), buf, len(buf)))
    return buf.raw[:n].decode()


def run(cfg: Cfg, model: Model, elites, out_path: str, count_out: str) -> int:
    """run(), src/screen.zig:257-343: screen, write the promoted and count files."""
    surv, total = screen(cfg, model, elites)
    if cfg.flags & _lib.FLAG_AS_SHIPPED:
        surv = surv[:0]
    with open(out_path, "w") as f:
        for r in surv:
            f.write(format_survivor(r, cfg.flags))
    with open(count_out, "w") as f:
        f.write(f"{total}\n")
    return total


def screen_device(cfg: Cfg, model: Model, elites_dev, out_dev, result_dev, stream=None) -> None:
    """Enqueue the screen on device buffers owned by torch.

    elites_dev: uint8 CUDA tensor holding n GENOME_DTYPE records (n*152 bytes);
    out_dev: uint8 CUDA tensor with room for min(keep, lambda) survivors;
    result_dev: int64/uint64 CUDA tensor of 4 words (count, screened, error
    bits, items). ``stream`` defaults to torch's current stream.
    """
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    ne = elites_dev.numel() // GENOME_DTYPE.itemsize
    keep_n = min(int(cfg.keep), int(cfg.lambda_))
    if out_dev.numel() < keep_n * SURVIVOR_DTYPE.itemsize or result_dev.numel() < 4:
        raise ValueError("output buffers too small")
    c = cfg.c()
    fn = lib().csx_screen_full_device if isinstance(model, ModelFull) else lib().csx_screen_device
    check(fn(ctypes.byref(c), ctypes.byref(model.c), elites_dev.data_ptr(), ne, out_dev.data_ptr(), keep_n,
             result_dev.data_ptr(), ctypes.c_void_p(stream.cuda_stream)), "screen_device")


def survivors_from_bytes(raw: np.ndarray, n: int) -> np.ndarray:
    return np.frombuffer(np.ascontiguousarray(raw).tobytes()[: n * SURVIVOR_DTYPE.itemsize],
                         dtype=SURVIVOR_DTYPE, count=n)


def last_run_info() -> dict:
    """Shape and (with FLAG_STAGE_TIMES) stage times of the last screen call."""
    info = _lib.CsxRunInfo()
    check(lib().csx_last_run_info(ctypes.byref(info)), "last_run_info")
    return {name: getattr(info, name) for name, _ in info._fields_}


def limits() -> Tuple[int, int]:
    k = ctypes.c_uint64(0)
    e = ctypes.c_uint64(0)
    lib().csx_limits(ctypes.byref(k), ctypes.byref(e))
    return int(k.value), int(e.value)


__all__ = ["Model", "ModelFull", "Cfg", "load_model", "parse_model_text", "screen", "run", "format_survivor",
           "screen_device", "survivors_from_bytes", "limits", "last_run_info", "VALID_N", "NTOT", "SURVIVOR_DTYPE"]
