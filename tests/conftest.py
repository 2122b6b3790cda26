import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_py
    oracle_py.build()
    oracle_py.load()
    return oracle_py


@pytest.fixture(scope="session")
def lib():
    """The product library; building it is the build step's job, so a missing
    library is an error here, not a skip."""
    import dynamicradiancevolume_gb300 as drv
    return drv.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    return torch.device("cuda:0")
