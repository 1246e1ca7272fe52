import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as xo
    xo.build()
    return xo


@pytest.fixture(scope="session")
def ref_lib(oracle):
    """The reference's own code compiled from its sources (oracle/_ref);
    skipped where the reference tree is absent (e.g. the GPU machine)."""
    if oracle.ref_lib() is None:
        oracle.build_ref()
    r = oracle.ref_lib()
    if r is None:
        pytest.skip("reference sources not present; golden fixtures cover this")
    return r


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from xdg_gb300 import _lib
    _lib.load()
    return torch
