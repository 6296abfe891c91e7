import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "bec-simulation_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libsbec kernels)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def libsbec():
    """Build (if stale) and load libsbec.so."""
    import build as sbec_build  # bec-simulation_gb300/build.py

    sbec_build.build()
    import spinorbec

    return spinorbec.load()


@pytest.fixture(scope="session")
def gpu(libsbec):
    import spinorbec

    if spinorbec.device_count() < 1:
        pytest.fail("GPU test selected but no CUDA device is visible")
    return True
