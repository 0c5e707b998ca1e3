import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "matflat_cases.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def cases(golden, prefix):
    """Case keys (without the trailing field) under a family prefix such as 'lu_d/'."""
    return sorted({k.rsplit("/", 1)[0] for k in golden if k.startswith(prefix)})


@pytest.fixture(scope="session")
def mf():
    """The CUDA library, built if needed; the tests that use it are marked gpu."""
    from matflat_gb300 import build
    build.build()
    import matflat_gb300
    matflat_gb300.context()
    return matflat_gb300
