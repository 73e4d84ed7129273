import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: long-running case")


def rel_l2(a, b):
    """Relative L2 error of a against reference b (over any number of fields)."""
    a = [np.asarray(x) for x in (a if isinstance(a, (list, tuple)) else [a])]
    b = [np.asarray(x) for x in (b if isinstance(b, (list, tuple)) else [b])]
    num = sum(float(np.sum(np.abs(x.astype(np.complex128) - y) ** 2)) for x, y in zip(a, b))
    den = sum(float(np.sum(np.abs(y) ** 2)) for y in b)
    return np.sqrt(num / den) if den > 0 else np.sqrt(num)


@pytest.fixture(scope="session")
def specns_lib():
    """The built CUDA library (built on demand; never a CPU fallback)."""
    from speccodelib_gb300 import build, _lib
    build.build()
    return _lib.load()
