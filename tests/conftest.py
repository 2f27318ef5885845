import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

EPS = float(np.finfo(np.float64).eps)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    O.set_blas_threads(1)
    return O


@pytest.fixture(scope="session")
def ctx():
    import paraht_gb300 as ph

    c = ph.Context(0)
    yield c
    c.close()
