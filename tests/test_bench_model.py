"""bench.py's algorithmic count for the roofline line (CPU): the full
synthesis per candidate with and without a linear tail, the pruning form's
count, and which surfaces carry a tail."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_full_synthesis_counts():
    import bench

    assert bench.full_synth_ops(True) == 1760.0
    # the tail's 0.99 x 26 crossover draws and 0.01 x 13 immigrant draws (x 20)
    # and its 13 genes (x 5) and 13 FMA (x 2) drop out
    assert bench.full_synth_ops(False) == pytest.approx(1760.0 - 25.87 * 20 - 13 * 7)


def test_pruning_count_scales_with_the_queue():
    import bench

    base = bench.prune_ops(0.0, False)
    assert base == pytest.approx(bench.PRUNE_DRAWS * 20 + 0.99 * 72)
    assert bench.prune_ops(0.02, False) - base == pytest.approx(0.02 * bench.full_synth_ops(False))
    assert bench.prune_ops(0.02, True) - base == pytest.approx(0.02 * 1760.0)


def test_which_surfaces_have_a_tail(csx):
    import bench
    from codec_arena_gb300 import screen, workloads as wl

    assert not bench.has_tail(screen.Model.from_compact(wl.surrogate_161()))
    assert not bench.has_tail(screen.Model.from_compact(wl.seeded_normal_model(seed=2)))
    w = np.random.default_rng(5).normal(0, 3, 166).astype(np.float32)
    assert bench.has_tail(screen.Model.from_compact(w))
