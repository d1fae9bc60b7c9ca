import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def engine():
    """The engine package with its library built in-tree."""
    from dedispersion_gb300 import build as b
    b.build()
    import dedispersion_gb300 as dd
    return dd


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def ref(oracle):
    h = oracle.reference()
    if h is None:
        pytest.skip("reference sources not available: oracle/_ref not built")
    return h


@pytest.fixture(scope="session")
def gpu(engine):
    # GPU tests fail (not skip) without a device: a skipped parity test
    # must never read as a pass on a GPU machine.
    assert engine.device_count() >= 1, "GPU tests need a CUDA device"
    return engine
