/*
 * csx_bench.h — measurement helpers (libcsx_bench.so), used by bench.py to
 * measure the roofline denominators of the integer/FP32-issue-bound screen on
 * the GPU it runs on. No reference counterpart: the reference publishes only
 * a hand-measured candidates/s figure (docs/SCALE.md:26).
 */
#ifndef CSX_BENCH_H
#define CSX_BENCH_H

#ifdef __cplusplus
extern "C" {
#endif

/* kind 0: integer ALU (shift/xor/add) lane-ops/s; 1: IMAD lane-ops/s;
 * 2: FFMA lane-ops/s; 3: splitmix64 outputs/s; 4: DFMA (FP64) lane-ops/s
 * (the ridge refit's normal equations). Returns 0 or a negative
 * csx status. Runs on the current device, default stream, synchronously. */
int csx_bench_issue_rate(int kind, double *per_second);

#ifdef __cplusplus
}
#endif
#endif
