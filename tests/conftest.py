import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build(with_ref=False)
    return oracle.Oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle
    oracle.build(with_ref=True)
    if not oracle.ref_available():
        pytest.skip("reference sources not present (only in the development checkout)")
    return oracle.Reference()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(scope="session")
def gpu():
    """A library context on cuda:0.  The CUDA library is the only path: a
    missing library or device is an error on a GPU machine, not a skip."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device in this environment")
    from centre_gb300 import build as B
    B.build()
    from centre_gb300.api import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
