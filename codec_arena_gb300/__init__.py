"""GB300-native screen funnel of codec-arena (src/screen.zig).

Modules:
  screen   Model / load_model / Cfg / run / screen / screen_device (the path)
  genome   genome parse / format (src/genome.zig)
  workloads  seeded synthetic elites and surrogate surfaces
  build    in-tree nvcc build of libcsx_screen.so and bin/arena
  cli      the `arena screen` verb
"""
from ._lib import NG, NR, NTOT, CsxError  # noqa: F401

__version__ = "0.1.0"
