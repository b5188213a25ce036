// arena_main.cpp — drop-in `arena` binary for brain/evolve.py's --zig flag.
//
// `arena screen ...` runs the GPU screen (src/main.zig:98-101 dispatch,
// :156-218 screenCmd). Every other verb (eval, psnr, msssimcheck, debug) is
// the reference's CPU referee and is handed unchanged to the binary named by
// CSX_ARENA_REAL, so one --zig path serves the whole generation loop.
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "csx_screen.h"

int main(int argc, char **argv) {
    if (argc >= 2 && std::strcmp(argv[1], "screen") == 0) {
        const int rc = csx_screen_cli(argc - 2, const_cast<const char *const *>(argv + 2));
        return rc == CSX_OK ? 0 : 1;
    }
    const char *real = std::getenv("CSX_ARENA_REAL");
    if (real && *real) {
        argv[0] = const_cast<char *>(real);
        execv(real, argv);
        std::perror("arena: exec CSX_ARENA_REAL");
        return 127;
    }
    std::fprintf(stderr,
                 "arena (GB300 screen) — verbs:\n"
                 "  screen --model FILE --elites POPFILE --out POPFILE --count-out FILE\n"
                 "         --lambda N --keep K --seed S [--threads T] [--sigma F] [--jump F] [--imm F]\n"
                 "         [--compat-29] [--as-shipped] [--parse-v6-fix] [--exact-all]\n"
                 "other verbs run the reference binary named by CSX_ARENA_REAL\n");
    return 2;
}
