import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libnbkdt kernels)")


@pytest.fixture(scope="session")
def port_built():
    import oracle
    oracle.build(ref=False)
    return True


@pytest.fixture(scope="session")
def ref_built():
    """The reference compiled from its own sources; only where its checkout exists."""
    import oracle
    src = oracle.ref_src()
    if not oracle.ref_present(src):
        pytest.skip("reference checkout not present on this machine")
    oracle.build(ref=True, ref_src=src)
    return True


@pytest.fixture(scope="session")
def lib_built():
    from nbodylib_gb300 import _build
    return _build.build()


@pytest.fixture(scope="session")
def gpu(lib_built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return True
