"""MatrixMarket input helpers and the driver's problematic-DOF selection
(tests/linear_solve.cpp:395-429), on CPU."""
import os

import numpy as np


def test_matrix_roundtrip_and_canonical_layout(tmp_path, built):
    import scipy.io
    import scipy.sparse as sp
    from lss import io
    rng = np.random.default_rng(0)
    A = sp.random(50, 50, density=0.1, random_state=1, format="coo")
    A = (A + A.T + sp.eye(50) * 5).tocoo()
    # duplicates and unsorted entries in the file
    rows = np.concatenate([A.row, A.row[:5]])
    cols = np.concatenate([A.col, A.col[:5]])
    vals = np.concatenate([A.data, rng.standard_normal(5)])
    D = sp.coo_matrix((vals, (rows, cols)), shape=A.shape)
    p = os.path.join(tmp_path, "A.mtx")
    scipy.io.mmwrite(p, D)
    B = io.read_matrix(p)
    assert B.format == "csc" and B.has_canonical_format
    assert abs(B - D.tocsc()).max() < 1e-12


def test_vector_and_problematic_dofs(tmp_path, built):
    import scipy.io
    from lss import io
    info = np.array([0.5, 2.0, -1.0, 3.0, 2.0])
    p = os.path.join(tmp_path, "p.mtx")
    scipy.io.mmwrite(p, info.reshape(-1, 1))
    v = io.read_vector(p, n=5)
    np.testing.assert_array_equal(v, info)
    np.testing.assert_array_equal(io.problematic_dofs(v, 1.9), [1, 3, 4])
    np.testing.assert_array_equal(io.problematic_dofs(v, 1.9, less_than=True), [0, 2])
    np.testing.assert_array_equal(io.problematic_dofs(v, 2.0), [3])  # strict, as the driver


def test_reference_fixture_reads(built):
    from conftest import GOLDEN, load_npz_matrix
    A = load_npz_matrix(os.path.join(GOLDEN, "A_contact.npz"))
    assert A.shape[0] == A.shape[1] and A.nnz > 0
