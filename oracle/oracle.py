"""ctypes binding of the CPU oracle (libcsx_oracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm as the checker. The product path
never imports this module.

Struct layouts equal the product's csx_* structs, so results compare as numpy
record arrays of the same dtype.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build as _build  # noqa: E402

NTOT = 29
GENOME_DTYPE = np.dtype({"names": ["id", "pa", "pb", "gen", "tribe", "g", "reserved"],
                         "formats": ["<u8", "<u8", "<u8", "<u4", "<u4", ("<f4", NTOT), "<u4"],
                         "offsets": [0, 8, 16, 24, 28, 32, 148], "itemsize": 152})
SURVIVOR_DTYPE = np.dtype({"names": ["score", "tribe", "pa", "pb", "stream", "index", "draw", "g",
                                     "reserved"],
                           "formats": ["<f4", "<u4", "<u8", "<u8", "<u8", "<u8", "<u8", ("<f4", NTOT),
                                       "<u4"],
                           "offsets": [0, 4, 8, 16, 24, 32, 40, 48, 164], "itemsize": 168})

FLAG_AS_SHIPPED = 0x1
FLAG_PARSE_V6_FIX = 0x4


class OrcModel(ctypes.Structure):
    _fields_ = [("w0", ctypes.c_float), ("w_lin", ctypes.c_float * NTOT),
                ("w_quad", ctypes.c_float * 256)]


FULL_NF = 465  # compact length of the full quadratic surface (csx_oracle.h)


class OrcModelFull(ctypes.Structure):
    _fields_ = [("w0", ctypes.c_float), ("w_lin", ctypes.c_float * NTOT),
                ("w_quad", ctypes.c_float * 435)]


class OrcCfg(ctypes.Structure):
    _fields_ = [("lambda_", ctypes.c_uint64), ("keep", ctypes.c_uint64), ("seed", ctypes.c_uint64),
                ("threads", ctypes.c_uint64), ("sigma", ctypes.c_float), ("jump_p", ctypes.c_float),
                ("imm_p", ctypes.c_float), ("flags", ctypes.c_uint32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        l = ctypes.CDLL(path)
        l.orc_splitmix_next.restype = ctypes.c_uint64
        l.orc_splitmix_next.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
        l.orc_stream_seed.restype = ctypes.c_uint64
        l.orc_stream_seed.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        l.orc_model_from_compact.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                                             ctypes.POINTER(OrcModel)]
        l.orc_model_parse.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_float),
                                      ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        l.orc_score.restype = ctypes.c_float
        l.orc_score.argtypes = [ctypes.POINTER(OrcModel), ctypes.c_void_p]
        l.orc_score_f64.restype = ctypes.c_double
        l.orc_score_f64.argtypes = [ctypes.POINTER(OrcModel), ctypes.c_void_p]
        l.orc_parse_line.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_void_p]
        l.orc_elites_parse.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        l.orc_candidate.argtypes = [ctypes.POINTER(OrcCfg), ctypes.POINTER(OrcModel), ctypes.c_void_p,
                                    ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
                                    ctypes.POINTER(ctypes.c_uint64)]
        l.orc_stream_dump.argtypes = [ctypes.POINTER(OrcCfg), ctypes.POINTER(OrcModel), ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p]
        l.orc_screen.argtypes = [ctypes.POINTER(OrcCfg), ctypes.POINTER(OrcModel), ctypes.c_void_p,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                                 ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        l.orc_model_full_from_compact.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                                                  ctypes.POINTER(OrcModelFull)]
        l.orc_score_full.restype = ctypes.c_float
        l.orc_score_full.argtypes = [ctypes.POINTER(OrcModelFull), ctypes.c_void_p]
        l.orc_score_full_f64.restype = ctypes.c_double
        l.orc_score_full_f64.argtypes = [ctypes.POINTER(OrcModelFull), ctypes.c_void_p]
        l.orc_candidate_full.argtypes = [ctypes.POINTER(OrcCfg), ctypes.POINTER(OrcModelFull), ctypes.c_void_p,
                                         ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
                                         ctypes.POINTER(ctypes.c_uint64)]
        l.orc_screen_full.argtypes = [ctypes.POINTER(OrcCfg), ctypes.POINTER(OrcModelFull), ctypes.c_void_p,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                                      ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        l.orc_walk.restype = ctypes.c_uint64
        l.orc_walk.argtypes = [ctypes.POINTER(OrcCfg), ctypes.c_uint64, ctypes.c_uint64,
                               ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
        _lib = l
    return _lib


def cfg(lambda_, keep, seed, threads=4, sigma=0.12, jump_p=0.02, imm_p=0.01, flags=0) -> OrcCfg:
    return OrcCfg(int(lambda_), int(keep), int(seed), int(threads), float(sigma), float(jump_p),
                  float(imm_p), int(flags))


def model_from_compact(w):
    w = np.ascontiguousarray(w, dtype=np.float32)
    m = OrcModel()
    rc = lib().orc_model_from_compact(w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(w),
                                      ctypes.byref(m))
    if rc:
        raise ValueError(f"orc_model_from_compact: {rc}")
    return m


def model_full_from_compact(w):
    """The full quadratic surface (465 compact floats; csx_oracle.h)."""
    w = np.ascontiguousarray(w, dtype=np.float32)
    m = OrcModelFull()
    rc = lib().orc_model_full_from_compact(w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(w),
                                           ctypes.byref(m))
    if rc:
        raise ValueError(f"orc_model_full_from_compact: {rc}")
    return m


def _full(m) -> bool:
    return isinstance(m, OrcModelFull)


def model_parse(text: str) -> np.ndarray:
    b = text.encode()
    w = (ctypes.c_float * 166)()
    n = ctypes.c_int(0)
    rc = lib().orc_model_parse(b, len(b), w, 166, ctypes.byref(n))
    if rc:
        raise ValueError(f"orc_model_parse: {rc}")
    return np.array(w[: n.value], dtype=np.float32)


def score(m, g) -> np.float32:
    g = np.ascontiguousarray(g, dtype=np.float32)
    f = lib().orc_score_full if _full(m) else lib().orc_score
    return np.float32(f(ctypes.byref(m), g.ctypes.data))


def score_f64(m, g) -> float:
    g = np.ascontiguousarray(g, dtype=np.float32)
    f = lib().orc_score_full_f64 if _full(m) else lib().orc_score_f64
    return float(f(ctypes.byref(m), g.ctypes.data))


def parse_line(line: str, flags: int = 0):
    b = line.encode()
    out = np.zeros(1, dtype=GENOME_DTYPE)
    rc = lib().orc_parse_line(b, len(b), flags, out.ctypes.data)
    if rc < 0:
        raise ValueError(f"orc_parse_line: {rc}")
    return out[0] if rc == 1 else None


def elites_parse(text: str, flags: int = 0) -> np.ndarray:
    b = text.encode()
    n = ctypes.c_int(0)
    lib().orc_elites_parse(b, len(b), flags, None, 0, ctypes.byref(n))
    out = np.zeros(max(1, n.value), dtype=GENOME_DTYPE)
    lib().orc_elites_parse(b, len(b), flags, out.ctypes.data, n.value, ctypes.byref(n))
    return out[: n.value]


def stream_dump(c: OrcCfg, m, elites, t: int, n: int) -> np.ndarray:
    e = np.ascontiguousarray(elites, dtype=GENOME_DTYPE)
    out = np.zeros(max(1, n), dtype=SURVIVOR_DTYPE)
    lib().orc_stream_dump(ctypes.byref(c), ctypes.byref(m), e.ctypes.data, len(e), t, n, out.ctypes.data)
    return out[:n]


def candidate(c: OrcCfg, m, elites, t: int, draw: int):
    e = np.ascontiguousarray(elites, dtype=GENOME_DTYPE)
    out = np.zeros(1, dtype=SURVIVOR_DTYPE)
    nxt = ctypes.c_uint64(0)
    f = lib().orc_candidate_full if _full(m) else lib().orc_candidate
    f(ctypes.byref(c), ctypes.byref(m), e.ctypes.data, len(e), t, draw, out.ctypes.data, ctypes.byref(nxt))
    return out[0], int(nxt.value)


def screen(c: OrcCfg, m, elites, cpu_threads: int = 0):
    """run() with the intended merge: (survivors, screened)."""
    e = np.ascontiguousarray(elites, dtype=GENOME_DTYPE)
    cap = int(min(c.keep, c.lambda_))
    out = np.zeros(max(1, cap), dtype=SURVIVOR_DTYPE)
    n = ctypes.c_uint64(0)
    scr = ctypes.c_uint64(0)
    f = lib().orc_screen_full if _full(m) else lib().orc_screen
    rc = f(ctypes.byref(c), ctypes.byref(m), e.ctypes.data, len(e), int(cpu_threads),
           out.ctypes.data, cap, ctypes.byref(n), ctypes.byref(scr))
    if rc:
        raise ValueError(f"orc_screen: {rc}")
    return out[: n.value], int(scr.value)


def walk(c: OrcCfg, t: int, start: int, end: int):
    nxt = ctypes.c_uint64(0)
    n = lib().orc_walk(ctypes.byref(c), t, start, end, ctypes.byref(nxt))
    return int(n), int(nxt.value)
