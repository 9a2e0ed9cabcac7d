import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.lib()
    oracle.set_blas_threads(1)
    return oracle


@pytest.fixture(scope="session")
def ooc():
    import oocdag_gb300

    oocdag_gb300.load()
    return oocdag_gb300


@pytest.fixture(scope="session")
def handle(ooc):
    if not gpu_available():
        pytest.skip("no GPU")
    h = ooc.Handle(0)
    yield h
    h.close()
