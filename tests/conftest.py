import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _build_lib():
    from eikonalxx_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import Reference
    try:
        return Reference()
    except (FileNotFoundError, RuntimeError) as e:
        pytest.skip(f"reference build unavailable: {e}")


@pytest.fixture(scope="session")
def lib():
    _build_lib()
    import eikonalxx_gb300 as ex
    return ex.load()


@pytest.fixture(scope="session")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _build_lib()
    import eikonalxx_gb300 as ex
    c = ex.Context(0)
    yield c
    c.close()


def random_slowness(rng, shape, vmin=2000.0, vmax=6000.0, dtype=np.float64):
    return (1.0 / rng.uniform(vmin, vmax, size=shape)).astype(dtype)
