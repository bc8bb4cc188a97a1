import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_cpu.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN, allow_pickle=False))


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle, build

    build(with_ref=False)
    return Oracle()


@pytest.fixture(scope="session")
def built_lib():
    from randomwalk_nmr_gb300 import build

    return build.build()


@pytest.fixture()
def engine(built_lib):
    """A fresh engine context on cuda:0 (GPU tests only; fails loudly without a GPU)."""
    from randomwalk_nmr_gb300 import Engine

    e = Engine(0)
    yield e
    e.close()


def dfactor(rho, res=1.0, d0=2.5):
    """Walker::computeDecreaseFactor (Walker/walker.h:203-209)."""
    return 1.0 - (2.0 / 3.0) * ((np.asarray(rho, dtype=np.float64) * res) / (d0 * 1e03))
