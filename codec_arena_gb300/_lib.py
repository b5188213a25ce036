"""ctypes binding of ``include/csx_screen.h`` (libcsx_screen.so).

The library is built in-tree by ``codec_arena_gb300.build``. Loading fails
loudly when it is missing: there is no CPU fallback for the screen.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

NG = 23
NR = 6
NTOT = 29

OK = 0
ERR_BAD_MODEL = -1
ERR_NEED_TWO_ELITES = -2
ERR_BAD_ARGS = -3
ERR_PARSE = -4
ERR_IO = -5
ERR_LIMIT = -6
ERR_CUDA = -7
ERR_NO_DEVICE = -8
ERR_OOM = -9
ERR_DEVICE_STATE = -10

FLAG_AS_SHIPPED = 0x1
FLAG_OUTPUT_29 = 0x2
FLAG_PARSE_V6_FIX = 0x4
FLAG_EXACT_ALL = 0x8
FLAG_STAGE_TIMES = 0x10
FLAG_TC_BF16 = 0x20
FLAG_TC_FP16 = 0x40
FLAG_NO_PRUNE = 0x80
FLAG_PRUNE_FFMA = 0x100

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libcsx_screen.so")

_f32 = ctypes.c_float
_u32 = ctypes.c_uint32
_u64 = ctypes.c_uint64


class CsxModel(ctypes.Structure):
    _fields_ = [("w0", _f32), ("w_lin", _f32 * NTOT), ("w_quad", _f32 * 256)]


class CsxGenome(ctypes.Structure):
    _fields_ = [("id", _u64), ("pa", _u64), ("pb", _u64), ("gen", _u32), ("tribe", _u32),
                ("g", _f32 * NTOT), ("reserved", _u32)]


class CsxCfg(ctypes.Structure):
    _fields_ = [("lambda_", _u64), ("keep", _u64), ("seed", _u64), ("threads", _u64),
                ("sigma", _f32), ("jump_p", _f32), ("imm_p", _f32), ("flags", _u32)]


class CsxSurvivor(ctypes.Structure):
    _fields_ = [("score", _f32), ("tribe", _u32), ("pa", _u64), ("pb", _u64), ("stream", _u64),
                ("index", _u64), ("draw", _u64), ("g", _f32 * NTOT), ("reserved", _u32)]


class CsxRunInfo(ctypes.Structure):
    _fields_ = [("launches", _u32), ("screen_ctas", _u32), ("segments", _u64), ("seg_draws", _u64),
                ("item_cands", _u64), ("items", _u64), ("ms_prep", _f32), ("ms_items", _f32),
                ("ms_screen", _f32), ("ms_merge", _f32), ("ms_regen", _f32), ("ms_total", _f32),
                ("exact_evals", _u64)]


# numpy views with the same layout (bulk conversion without per-field ctypes)
GENOME_DTYPE = np.dtype({"names": ["id", "pa", "pb", "gen", "tribe", "g", "reserved"],
                         "formats": ["<u8", "<u8", "<u8", "<u4", "<u4", ("<f4", NTOT), "<u4"],
                         "offsets": [0, 8, 16, 24, 28, 32, 148], "itemsize": 152})
SURVIVOR_DTYPE = np.dtype({"names": ["score", "tribe", "pa", "pb", "stream", "index", "draw", "g",
                                     "reserved"],
                           "formats": ["<f4", "<u4", "<u8", "<u8", "<u8", "<u8", "<u8", ("<f4", NTOT),
                                       "<u4"],
                           "offsets": [0, 4, 8, 16, 24, 32, 40, 48, 164], "itemsize": 168})

assert ctypes.sizeof(CsxGenome) == GENOME_DTYPE.itemsize == 152
assert ctypes.sizeof(CsxSurvivor) == SURVIVOR_DTYPE.itemsize == 168
assert ctypes.sizeof(CsxCfg) == 48
assert ctypes.sizeof(CsxRunInfo) == 72
assert ctypes.sizeof(CsxModel) == 4 * (1 + NTOT + 256)

# Every entry point of include/csx_screen.h with its ctypes signature.
SIGNATURES = {
    "csx_abi_version": (ctypes.c_int, []),
    "csx_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "csx_cfg_default": (None, [ctypes.POINTER(CsxCfg)]),
    "csx_model_from_compact": (ctypes.c_int, [ctypes.POINTER(_f32), ctypes.c_int,
                                              ctypes.POINTER(CsxModel)]),
    "csx_model_parse": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_f32),
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "csx_genome_parse_line": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t, _u32,
                                             ctypes.POINTER(CsxGenome)]),
    "csx_elites_parse": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t, _u32, ctypes.c_void_p,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "csx_genome_format_line": (ctypes.c_int, [ctypes.POINTER(CsxGenome), ctypes.c_char_p,
                                              ctypes.c_size_t]),
    "csx_survivor_format_line": (ctypes.c_int, [ctypes.c_void_p, _u32, ctypes.c_char_p,
                                                ctypes.c_size_t]),
    "csx_screen": (ctypes.c_int, [ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModel), ctypes.c_void_p,
                                  ctypes.c_int, ctypes.c_void_p, _u64, ctypes.POINTER(_u64),
                                  ctypes.POINTER(_u64)]),
    "csx_screen_range": (ctypes.c_int, [ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModel), ctypes.c_void_p,
                                        ctypes.c_int, _u64, _u64, ctypes.c_void_p, _u64, ctypes.POINTER(_u64),
                                        ctypes.POINTER(_u64)]),
    "csx_screen_items": (ctypes.c_int, [ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModel), ctypes.c_void_p,
                                        ctypes.c_int, _u32, _u32, ctypes.c_void_p, _u64, ctypes.POINTER(_u64),
                                        ctypes.POINTER(_u64)]),
    "csx_screen_device": (ctypes.c_int, [ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModel),
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, _u64,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "csx_screen_device_noalloc": (ctypes.c_int, [ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModel),
                                                 ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, _u64,
                                                 ctypes.c_void_p, ctypes.c_void_p]),
    "csx_screen_cli": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]),
    "csx_limits": (ctypes.c_int, [ctypes.POINTER(_u64), ctypes.POINTER(_u64)]),
    "csx_last_run_info": (ctypes.c_int, [ctypes.POINTER(CsxRunInfo)]),
}

# include/csx_surrogate.h (same library); device pointers and the stream as void*.
_vp, _i64, _int = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
SURROGATE_SIGNATURES = {
    "csx_sg_workspace_bytes": (_u64, [_int]),
    "csx_sg_forward": (_int, [_vp, _int, _vp, _i64, _int, _int, _vp, _vp]),
    "csx_sg_forward_f64": (_int, [_vp, _int, _vp, _i64, _int, _vp, _vp]),
    "csx_sg_backward": (_int, [_vp, _int, _vp, _i64, _int, _int, _vp, _vp, _vp, _vp, _vp]),
    "csx_sg_backward_coef_f64": (_int, [_int, _vp, _i64, _int, _vp, _vp, _vp, _vp]),
    "csx_sg_normal_equations": (_int, [_int, _vp, _i64, _int, _vp, _vp, _vp, _vp, _vp]),
    "csx_sg_ridge_solve": (_int, [_int, _vp, _vp, ctypes.c_double, _vp, _vp, _vp, _vp]),
    "csx_sg_ascend": (_int, [_vp, _int, _vp, _i64, _int, _f32, _int, _vp, _vp]),
}
SIGNATURES.update(SURROGATE_SIGNATURES)

MAX_ISLANDS = 64


class CsxBatchTune(ctypes.Structure):
    _fields_ = [("item_cands", _u32), ("seg_cands", _u32), ("ctas_per_sm", _u32), ("reserved", _u32)]


class CsxBatchInfo(ctypes.Structure):
    _fields_ = [("islands", _u32), ("launches", _u32), ("screen_ctas", _u32), ("graph_nodes", _u32),
                ("ms_capture", _f32), ("ms_device", _f32)]


SIGNATURES.update({
    "csx_screen_batch": (_int, [_int, ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModel), _vp,
                                ctypes.POINTER(_int), ctypes.POINTER(CsxBatchTune), _vp, ctypes.POINTER(_u64),
                                ctypes.POINTER(_u64)]),
    "csx_screen_batch_device": (_int, [_int, ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModel), _vp,
                                       ctypes.POINTER(_int), ctypes.POINTER(CsxBatchTune), _vp, _vp, _vp]),
    "csx_last_batch_info": (_int, [ctypes.POINTER(CsxBatchInfo)]),
    "csx_tc_score": (_int, [ctypes.POINTER(CsxModel), _int, _vp, _i64, _int, _vp, _vp, _vp]),
    "csx_score": (_int, [ctypes.POINTER(CsxModel), _vp, _i64, _int, _vp, _vp]),
})
TC_BF16, TC_FP16 = 1, 2

FULL_NF = 465  # compact length of the full quadratic surface (csx_screen.h)


class CsxModelFull(ctypes.Structure):
    _fields_ = [("w0", _f32), ("w_lin", _f32 * NTOT), ("w_quad", _f32 * 435)]


SIGNATURES.update({
    "csx_model_full_from_compact": (_int, [ctypes.POINTER(_f32), _int, ctypes.POINTER(CsxModelFull)]),
    "csx_screen_full": (_int, [ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModelFull), _vp, _int, _vp, _u64,
                               ctypes.POINTER(_u64), ctypes.POINTER(_u64)]),
    "csx_screen_full_range": (_int, [ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModelFull), _vp, _int, _u64, _u64,
                                     _vp, _u64, ctypes.POINTER(_u64), ctypes.POINTER(_u64)]),
    "csx_screen_full_device": (_int, [ctypes.POINTER(CsxCfg), ctypes.POINTER(CsxModelFull), _vp, _int, _vp,
                                      _u64, _vp, _vp]),
    "csx_score_full": (_int, [ctypes.POINTER(CsxModelFull), _vp, _i64, _int, _vp, _vp]),
})

SG_FP32, SG_BF16, SG_FP64 = 0, 1, 2

_lib = None


class CsxError(RuntimeError):
    """A non-zero status from the C ABI; ``.status`` holds the code."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        name = lib().csx_strerror(status).decode() if _lib is not None else str(status)
        super().__init__(f"{name}{': ' + what if what else ''} (status {status})")


def lib() -> ctypes.CDLL:
    """Load libcsx_screen.so once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run codec_arena_gb300.build.build() first "
                              "(the screen has no CPU fallback)")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(status: int, what: str = "") -> int:
    if status < 0:
        raise CsxError(status, what)
    return status
