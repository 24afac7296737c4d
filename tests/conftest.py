import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libvkhr_cuda.so")


@pytest.fixture(scope="session")
def oracle_lib():
    """The CPU oracle (built on first use; the checker, never the product)."""
    from oracle import oracle as O

    if not os.path.exists(O.LIB):
        O.build(with_reference=False)
    O.lib()
    return O


@pytest.fixture(scope="session")
def native_lib():
    """libvkhr_cuda.so loaded without touching the GPU (built if missing)."""
    from vkhr_gb300 import _native, build

    if not os.path.exists(_native.LIB_PATH):
        build.build(quiet=True)
    return _native.load()


@pytest.fixture(scope="session")
def ctx(native_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from vkhr_gb300 import _native

    c = _native.Context(0)
    yield c
    c.close()
