"""The reference-side binding: what `brain/evolve.py` needs to call the GPU
screen in process, without importing this package (only ctypes).

Copy this file next to `brain/evolve.py` and call `gpu_screen` where
`brain/evolve.py:431-454` runs `arena screen` as a subprocess. The structs are
those of `include/csx_screen.h`; the library path comes from `CSX_LIB` or
defaults to the in-tree build beside this file.
"""
import ctypes
import os

NTOT = 29


class Model(ctypes.Structure):
    _fields_ = [("w0", ctypes.c_float), ("w_lin", ctypes.c_float * NTOT), ("w_quad", ctypes.c_float * 256)]


class Genome(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("pa", ctypes.c_uint64), ("pb", ctypes.c_uint64), ("gen", ctypes.c_uint32),
                ("tribe", ctypes.c_uint32), ("g", ctypes.c_float * NTOT), ("reserved", ctypes.c_uint32)]


class Cfg(ctypes.Structure):
    _fields_ = [("lam", ctypes.c_uint64), ("keep", ctypes.c_uint64), ("seed", ctypes.c_uint64),
                ("threads", ctypes.c_uint64), ("sigma", ctypes.c_float), ("jump_p", ctypes.c_float),
                ("imm_p", ctypes.c_float), ("flags", ctypes.c_uint32)]


class Survivor(ctypes.Structure):
    _fields_ = [("score", ctypes.c_float), ("tribe", ctypes.c_uint32), ("pa", ctypes.c_uint64),
                ("pb", ctypes.c_uint64), ("stream", ctypes.c_uint64), ("index", ctypes.c_uint64),
                ("draw", ctypes.c_uint64), ("g", ctypes.c_float * NTOT), ("reserved", ctypes.c_uint32)]


csx = ctypes.CDLL(os.environ.get("CSX_LIB") or os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                           "libcsx_screen.so"))
csx.csx_strerror.restype = ctypes.c_char_p


def gpu_screen(weights, elites, screens, keep, seed, threads, sigma, jump=0.02, imm=0.01):
    """`arena screen` in process: compact surrogate weights, elites as
    evolve.py's dicts (id, gen, pa, pb, tribe, g[29]); returns the promoted
    genomes (34-token v6 fields, id and gen 0) and the screened count."""
    m = Model()
    w = (ctypes.c_float * len(weights))(*weights)
    assert csx.csx_model_from_compact(w, len(weights), ctypes.byref(m)) == 0
    el = (Genome * len(elites))()
    for i, g in enumerate(elites):
        el[i].id, el[i].gen, el[i].pa, el[i].pb, el[i].tribe = g["id"], g["gen"], g["pa"], g["pb"], g["tribe"]
        el[i].g[:] = g["g"]
    cfg = Cfg(screens, keep, seed, threads, sigma, jump, imm, 0)
    out = (Survivor * keep)()
    n, screened = ctypes.c_uint64(), ctypes.c_uint64()
    rc = csx.csx_screen(ctypes.byref(cfg), ctypes.byref(m), el, len(elites), out, keep,
                        ctypes.byref(n), ctypes.byref(screened))
    if rc != 0:
        raise RuntimeError(csx.csx_strerror(rc).decode())
    return [{"id": 0, "gen": 0, "pa": s.pa, "pb": s.pb, "tribe": s.tribe, "g": list(s.g)}
            for s in out[: n.value]], screened.value
