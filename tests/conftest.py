import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "cmc-cosmic_gb300"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gpulib():
    """The built in-tree libcmcgpu.so (building it first if needed)."""
    import cmcgpu

    cmcgpu.build()
    return cmcgpu


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build()
    return oracle
