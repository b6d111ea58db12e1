import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103) device and librsx.so")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def golden_1888():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "test1888.npz")))


@pytest.fixture(scope="session")
def golden_synth():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "synthetic_ref.npz")))
