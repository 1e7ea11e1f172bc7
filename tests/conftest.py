import os
import sys
from pathlib import Path

import pytest

pytest.register_assert_rewrite("gpu_helpers")

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")


@pytest.fixture(scope="session")
def built():
    """Builds the native library and the oracle once per session."""
    from kite_gb300.build import build
    import oracle as orc
    info = build()
    orc.build()
    return info


@pytest.fixture(scope="session")
def orc(built):
    import oracle as orc
    orc.lib()
    return orc


@pytest.fixture(scope="session")
def gpu(built):
    from kite_gb300 import gpu as g
    if g.device_count() < 1:
        pytest.fail("a GPU test ran without a visible CUDA device")
    return g
