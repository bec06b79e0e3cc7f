"""Input helpers of the reference's linear_solve driver for this path.

read_matrix / read_vector load MatrixMarket files (the reference's mats/*.mtx
fixtures and `-A` / `-b` / `-i` inputs) into the layout the solver takes:
compressed sparse columns with sorted indices and no duplicates (Eigen's
compressed StiffnessMatrix), and a dense vector.  problematic_dofs restates the
`-i` / `-t` / `--less_than` selection (tests/linear_solve.cpp:395-429) whose
result feeds Solver.set_problematic_dofs.
"""
from __future__ import annotations

import warnings

import numpy as np


def _mmread(path):
    import scipy.io
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", DeprecationWarning)  # scipy's spmatrix default change
        return scipy.io.mmread(path)


def read_matrix(path: str):
    """MatrixMarket matrix as a canonical scipy CSC matrix (float64)."""
    import scipy.sparse as sp
    A = sp.csc_matrix(_mmread(path), dtype=np.float64)
    A.sum_duplicates()
    A.sort_indices()
    return A


def read_vector(path: str, n: int | None = None) -> np.ndarray:
    """MatrixMarket vector (dense array or one-column coordinate file)."""
    v = _mmread(path)
    v = np.asarray(v.todense() if hasattr(v, "todense") else v, dtype=np.float64).ravel()
    if n is not None and v.size != n:
        raise ValueError(f"vector of size {v.size}, expected {n}")
    return v


def problematic_dofs(info, threshold: float, less_than: bool = False) -> np.ndarray:
    """DOFs i with info[i] > threshold (info[i] < threshold with less_than),
    ascending -- the set the driver passes to set_problematic_dofs."""
    info = np.asarray(info, dtype=np.float64).ravel()
    mask = info < threshold if less_than else info > threshold
    return np.nonzero(mask)[0].astype(np.int32)
