"""`arena screen` verb (src/main.zig:156-218) backed by the GPU screen.

    python -m codec_arena_gb300 screen --model FILE --elites POPFILE --out POPFILE \
        --count-out FILE --lambda N --keep K --seed S [--threads T] [--sigma F] \
        [--jump F] [--imm F] [--compat-29] [--as-shipped] [--parse-v6-fix] [--exact-all]

Flag parsing, file formats and error names follow the reference; the exit
status is 0 on success and 1 on any error, as a Zig `main` returning an error.
"""
from __future__ import annotations

import ctypes
import sys

from ._lib import lib


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    if not argv or argv[0] != "screen":
        sys.stderr.write(__doc__)
        return 2
    args = [a.encode() for a in argv[1:]]
    arr = (ctypes.c_char_p * max(1, len(args)))(*args)
    rc = lib().csx_screen_cli(len(args), arr)
    return 0 if rc == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
