"""Genome data model of the screen path (src/genome.zig), host side.

A genome is 23 effector genes and 6 regulator genes in [0, 1] plus lineage.
Arrays of genomes use ``GENOME_DTYPE`` (the ``csx_genome`` layout), with the
genes flattened in the order the screen reads them (src/screen.zig:240-241).
Parsing and formatting call the C ABI so that text -> f32 conversion is the
correctly rounded one the reference's ``std.fmt.parseFloat(f32, ...)`` does.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from ._lib import GENOME_DTYPE, NG, NR, NTOT, check, lib

NEW_GENE_LEGACY = 0.0  # src/genome.zig:106
REG_DEFAULT = 0.5


def clamp01(x: float) -> float:
    """src/genome.zig:292-294 (NaN maps to 1, as @min(1, NaN) does)."""
    if x != x:
        return 1.0
    return max(0.0, min(1.0, x))


def _to_record(g: _lib.CsxGenome) -> np.ndarray:
    return np.frombuffer(bytes(g), dtype=GENOME_DTYPE, count=1)[0]


def parse_line(line: str, v6_fix: bool = False) -> Optional[np.void]:
    """parseLine, src/genome.zig:116-188.

    Returns a ``GENOME_DTYPE`` record, ``None`` for a line that is not a genome
    (wrong token count or a comment) and raises ``CsxError`` on a malformed
    number. As written in the reference, a 34-token line keeps genes 16..21 at
    0.0; ``v6_fix=True`` reads them.
    """
    b = line.encode()
    g = _lib.CsxGenome()
    rc = lib().csx_genome_parse_line(b, len(b), _lib.FLAG_PARSE_V6_FIX if v6_fix else 0,
                                     ctypes.byref(g))
    if rc == 0:
        return None
    check(rc, "parseLine")
    return _to_record(g)


def load_elites_text(text: str, v6_fix: bool = False) -> np.ndarray:
    """The elites loop of src/main.zig:201-214: blank, '#' and bad lines skipped."""
    b = text.encode()
    flags = _lib.FLAG_PARSE_V6_FIX if v6_fix else 0
    n = ctypes.c_int(0)
    check(lib().csx_elites_parse(b, len(b), flags, None, 0, ctypes.byref(n)))
    out = np.zeros(max(n.value, 1), dtype=GENOME_DTYPE)
    check(lib().csx_elites_parse(b, len(b), flags, out.ctypes.data, n.value, ctypes.byref(n)))
    return out[: n.value]


def load_elites(path: str, v6_fix: bool = False) -> np.ndarray:
    with open(path, "r") as f:
        return load_elites_text(f.read(), v6_fix=v6_fix)


def format_line(rec) -> str:
    """formatLine, src/genome.zig:191-201 (34 tokens, genes to 4 decimals)."""
    g = _lib.CsxGenome()
    ctypes.memmove(ctypes.byref(g), np.asarray(rec, dtype=GENOME_DTYPE).tobytes(), ctypes.sizeof(g))
    buf = ctypes.create_string_buffer(1024)
    n = check(lib().csx_genome_format_line(ctypes.byref(g), buf, len(buf)))
    return buf.raw[:n].decode()


def make_genomes(genes, ids=None, tribes=None, gens=None) -> np.ndarray:
    """Build a ``GENOME_DTYPE`` array from an (n, 29) gene matrix."""
    genes = np.asarray(genes, dtype=np.float32)
    if genes.ndim != 2 or genes.shape[1] != NTOT:
        raise ValueError(f"genes must be (n, {NTOT})")
    n = genes.shape[0]
    out = np.zeros(n, dtype=GENOME_DTYPE)
    out["g"] = genes
    out["id"] = np.arange(n, dtype=np.uint64) if ids is None else np.asarray(ids, dtype=np.uint64)
    out["tribe"] = 0 if tribes is None else np.asarray(tribes, dtype=np.uint32)
    out["gen"] = 0 if gens is None else np.asarray(gens, dtype=np.uint32)
    return out


__all__ = ["NG", "NR", "NTOT", "NEW_GENE_LEGACY", "REG_DEFAULT", "GENOME_DTYPE", "clamp01",
           "parse_line", "load_elites", "load_elites_text", "format_line", "make_genomes"]
