"""Build recipe for the CPU oracle (test infrastructure).

Compiles ``oracle/csx_oracle.c`` into ``oracle/libcsx_oracle.so`` with
``-ffp-contract=off`` so each f32 multiply and add rounds on its own, as the
Zig reference's strict float mode does. Plain C: the same source builds on
x86-64 and aarch64 hosts.

The reference itself (Zig) cannot be compiled with the toolchains available,
so there is no ``oracle/_ref`` build; this restatement is the oracle.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libcsx_oracle.so")
SRC = os.path.join(HERE, "csx_oracle.c")

CFLAGS = ["-O3", "-std=gnu11", "-fPIC", "-shared", "-pthread",
          "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> str:
    """Compile the oracle if its source is newer than the library."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "csx_oracle.h")))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", *CFLAGS, "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
