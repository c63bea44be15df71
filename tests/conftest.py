import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "skewlinearalgebra.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libskewgpu.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    from oracle.build_oracle import build_oracle

    build_oracle()
    return O


@pytest.fixture(scope="session")
def skewgpu():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import skewgpu as sg

    return sg
