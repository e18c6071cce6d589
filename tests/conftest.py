import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (GB300); calls the CUDA library through the C ABI")
    # temporary files of the tests stay inside the repository (git-ignored)
    if not config.option.basetemp:
        config.option.basetemp = os.path.join(ROOT, "tests", ".tmp")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "reference_cpu.npz"))


@pytest.fixture(scope="session")
def lib_built():
    """Build the CUDA library (cross-compiles without a GPU) and the oracle."""
    from microsn_gb300 import build as B
    import oracle
    oracle.build()
    B.build()
    return True


@pytest.fixture(scope="session")
def ctx(lib_built):
    import torch
    import microsn_gb300 as mlc
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = mlc.Context(0)
    yield c
    c.close()
