import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def native():
    import lpmkokkos_gb300
    lpmkokkos_gb300.build()
    return lpmkokkos_gb300.lib()


@pytest.fixture(scope="session")
def ctx(native):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from lpmkokkos_gb300 import bve
    c = bve.Context(0)
    yield c
    c.close()
