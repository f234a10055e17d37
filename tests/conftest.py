import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests of the GPU library")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN, allow_pickle=False) as d:
        return {k: d[k] for k in d.files}


def csr_from(g, prefix):
    import scipy.sparse as sp
    shape = tuple(int(x) for x in g[prefix + "_shape"])
    # copies, so that no consumer can alter the session-wide fixture
    return sp.csr_array((g[prefix + "_data"].copy(), g[prefix + "_indices"].copy(), g[prefix + "_indptr"].copy()),
                        shape=shape)


def illc1850():
    """The reference's example matrix as shipped with scipy's tests, or None."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    path = os.path.join(os.path.dirname(sla.__file__), "tests", "propack_test_data.npz")
    if not os.path.exists(path):
        return None
    with np.load(path, allow_pickle=True) as data:
        return sp.csr_array(data["A_real"].item())


def mhd1280b():
    """The reference's complex example matrix (Examples/mhd1280b.cua) as
    shipped with scipy's tests, or None."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    path = os.path.join(os.path.dirname(sla.__file__), "tests", "propack_test_data.npz")
    if not os.path.exists(path):
        return None
    with np.load(path, allow_pickle=True) as data:
        return sp.csr_array(data["A_complex"].item())


def subspace_err(u1, u2):
    """max | |u1_i . u2_i| - 1 | over matched columns."""
    return float(np.max(np.abs(np.abs(np.sum(u1 * u2, axis=0)) - 1.0)))
