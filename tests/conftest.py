import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _product_built():
    """Builds libdrv_gb300.so (incremental: nothing to do when it is up to
    date), so that the suite also runs from a fresh checkout; a build that
    fails fails the session."""
    from dynamicradiancevolume_gb300 import build
    build.build()


@pytest.fixture(scope="session")
def oracle():
    import oracle_py
    oracle_py.build()
    oracle_py.load()
    return oracle_py


@pytest.fixture(scope="session")
def lib():
    """The product library (built by `_product_built`); a library that does
    not load is an error here, not a skip."""
    import dynamicradiancevolume_gb300 as drv
    return drv.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    return torch.device("cuda:0")
