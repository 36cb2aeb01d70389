import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def ddp():
    """The product package with its native library built."""
    from ddp_gb300 import build as B
    B.build()
    import ddp_gb300
    ddp_gb300.lib()
    return ddp_gb300


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    z = np.load(os.path.join(ROOT, "tests", "golden", "astar_ref.npz"))
    cases = {}
    for k in z.files:
        name, field = k.rsplit(".", 1)
        cases.setdefault(name, {})[field] = z[k]
    return cases


@pytest.fixture(scope="session")
def gpu(ddp):
    if ddp.lib().ddp_device_count() < 1:
        pytest.skip("no CUDA device")
    return ddp
