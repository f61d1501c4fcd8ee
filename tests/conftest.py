"""Shared pytest configuration.

Tests marked ``gpu`` need a CUDA GPU and the in-tree CUDA library; they call
the solvers through the C ABI and compare them with the FP64 oracle.  They fail
(never skip) when no GPU is present, so a silent fallback cannot pass them.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libseidart_gb300.so")


@pytest.fixture(scope="session")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("this test needs a CUDA GPU; run the CPU suite with -m 'not gpu'")
    from seidart_gb300 import build
    build.build()
    from seidart_gb300 import _lib
    _lib.lib()
    return torch.device("cuda:0")
