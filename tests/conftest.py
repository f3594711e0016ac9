import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) device")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build(with_reference=False)
    return oracle


@pytest.fixture(scope="session")
def xg():
    import xyce_gb300
    if not os.path.exists(xyce_gb300.LIB_PATH):
        xyce_gb300.build()
    return xyce_gb300
