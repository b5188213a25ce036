import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


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
