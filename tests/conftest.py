import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# The library prunes only generations large enough for pruning to pay (about
# 400 candidates per screen thread); the tests' generations are small, so they
# lower that floor to 0 and run the pruning kernels at every size.
# tests/test_gpu_screen.py::test_small_generations_take_the_unpruned_form
# checks the automatic choice.
os.environ.setdefault("CSX_PRUNE_MIN_CANDS", "0")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running GPU case")


@pytest.fixture(scope="session")
def csx():
    """The product library, built in-tree if needed."""
    from codec_arena_gb300 import build

    build.build()
    from codec_arena_gb300 import _lib

    return _lib.lib()


@pytest.fixture(scope="session")
def orc():
    import oracle  # noqa: F401  (oracle/oracle.py)

    oracle.lib()
    return oracle


def has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
