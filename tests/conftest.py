"""Test configuration: markers, import path and the GPU gate.

``-m gpu`` tests need a CUDA device and the built library; everything else runs on CPU.
"""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libetalon_gb300.so")
    config.addinivalue_line("markers", "slow: long CPU runs")


@pytest.fixture(scope="session")
def gpu():
    """The loaded library on a machine with a GPU; a GPU test fails loudly without one."""
    from etalon_gb300 import _lib

    _lib.lib()
    dev, name, sms = _lib.device_info()
    return {"device": dev, "name": name, "sms": sms}
