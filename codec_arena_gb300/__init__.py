"""GB300-native screen funnel of codec-arena (src/screen.zig).

Modules:
  screen     Model / load_model / Cfg / run / screen / screen_device /
             score_genes (the path; `streams=` screens a range of RNG streams)
  genome     genome parse / format (src/genome.zig)
  brain      brain/evolve.py's screen step in process, its file formats and
             search-counter bookkeeping
  islands    several islands screened in one graph launch
  autotune   tunables of the islands pipeline, timed and cached
  precision  the tensor-core (BF16 / FP16) scoring form
  surrogate  the differentiable surrogate: autograd, GPU ridge refit,
             gradient-guided mutation (brain/evolve.py:211-268)
  parallel   island seeds, stream ranges and survivor merges across ranks
  workloads  seeded synthetic elites, surfaces, islands and refit tables
  build      in-tree nvcc build of libcsx_screen.so, libcsx_bench.so, bin/arena
  cli        the `arena screen` verb
"""
from ._lib import NG, NR, NTOT, CsxError  # noqa: F401

__version__ = "0.2.0"
