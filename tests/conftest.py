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


@pytest.fixture(scope="session")
def golden_sasa():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "sasa_ref.npz")))


def sasa_dot_sets(golden, kind):
    """The reference's per-type dot sets of sasa_ref.npz as a list of (n_t, 4)."""
    d, s = golden[f"dots_{kind}"], golden[f"dots_{kind}_start"]
    return [d[s[t]:s[t + 1]] for t in range(len(s) - 1)]


def sasa_dot_map(golden, kind):
    """The same as one (n_types, stride, 4) map padded with -inf dots (the
    layout of the reference's OpenCL dots_map_, rsasa_cl_gpu_alg.cpp:72-86)."""
    import numpy as np
    sets = sasa_dot_sets(golden, kind)
    stride = max(len(x) for x in sets)
    m = np.full((len(sets), stride, 4), -np.inf, np.float32)
    for t, x in enumerate(sets):
        m[t, :len(x)] = x
    return m
