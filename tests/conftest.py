import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "local-stiff-solver_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__ as g
    g.build()
    return True


def load_npz_matrix(path):
    import scipy.sparse as sp
    z = np.load(path)
    n = len(z["indptr"]) - 1
    return sp.csc_matrix((z["data"], z["indices"], z["indptr"]), shape=(n, n))


@pytest.fixture(scope="session")
def golden():
    z = np.load(os.path.join(GOLDEN, "selection_golden.npz"))
    return {k: z[k] for k in z.files}


def reference_matrices():
    """The reference's example matrices available here: A_contact (committed),
    A_pq (generated by tests/golden/make_golden.py, not committed)."""
    out = {"A_contact": os.path.join(GOLDEN, "A_contact.npz")}
    big = os.path.join(GOLDEN, "_large", "A_pq.npz")
    if os.path.exists(big):
        out["A_pq"] = big
    return out
