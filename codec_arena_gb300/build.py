"""In-tree build of the screen funnel's native code (sm_103a only).

Produces, next to this file:
  * ``libcsx_screen.so`` — the C ABI of ``include/csx_screen.h`` (CUDA kernels
    and host code, cudart linked statically);
  * ``libcsx_bench.so`` — measurement kernels for bench.py (include/csx_bench.h);
  * ``bin/arena`` — a drop-in ``arena`` binary whose ``screen`` verb runs on the
    GPU and whose other verbs are handed to the reference binary named by
    ``CSX_ARENA_REAL``.

Translation units compile in parallel; nothing here needs cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcsx_screen.so")
BENCH_LIB = os.path.join(PKG, "libcsx_bench.so")
BIN_DIR = os.path.join(PKG, "bin")
ARENA = os.path.join(BIN_DIR, "arena")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]

UNITS = [  # (source, compiler, library)
    ("csx_screen.cu", "nvcc", LIB),
    ("csx_host.cpp", "g++", LIB),
    ("csx_surrogate.cu", "nvcc", LIB),
    ("csx_bench.cu", "nvcc", BENCH_LIB),
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _compile(src: str, kind: str, verbose: bool) -> str:
    os.makedirs(BUILD, exist_ok=True)
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cuh")] + [
        os.path.join(ROOT, "include", h) for h in ("csx_screen.h", "csx_surrogate.h", "csx_bench.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    if kind == "nvcc":
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-Xptxas", "-v" if verbose else "-O3", "-c", path, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", os.path.join(ROOT, "include"),
               "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    """Compile every translation unit (in parallel) and link the library and CLI."""
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose), UNITS))
    for lib_path in (LIB, BENCH_LIB):
        lib_objs = [o for o, u in zip(objs, UNITS) if u[2] == lib_path]
        newest = max(os.path.getmtime(o) for o in lib_objs)
        if not os.path.exists(lib_path) or os.path.getmtime(lib_path) < newest:
            tmp = lib_path + f".tmp{os.getpid()}"
            cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *lib_objs, "-lpthread"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
            os.replace(tmp, lib_path)
    os.makedirs(BIN_DIR, exist_ok=True)
    main_src = os.path.join(CSRC, "arena_main.cpp")
    if not os.path.exists(ARENA) or os.path.getmtime(ARENA) < max(os.path.getmtime(LIB),
                                                                   os.path.getmtime(main_src)):
        tmp = ARENA + f".tmp{os.getpid()}"
        cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), main_src, "-o", tmp,
               "-L", PKG, "-lcsx_screen", "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, ARENA)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
