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


@pytest.fixture(autouse=True)
def _fresh_plans(request):
    """Plans are keyed by array addresses, and torch reuses the addresses of freed tensors: the
    session context drops its plans after every test that used it, as the C ABI asks of callers
    that move on to an unrelated problem (lpm_bve_plan_invalidate)."""
    yield
    if "ctx" in request.fixturenames:
        request.getfixturevalue("ctx").invalidate()
