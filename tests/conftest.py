import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT / "rhizome_v24.15_gb300"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the engine through its C ABI")
    config.addinivalue_line("markers", "slow: long-running (full-size workloads)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def engine():
    """The CUDA engine; fails (does not skip) when the library or the device is missing."""
    import torch

    import gbsdf

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    gbsdf.load()
    return gbsdf
