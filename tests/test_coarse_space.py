"""The MAS coarse space (host only, through lss_coarse_space) against the
oracle's restatement of MASPreconditioner's coarse-space construction
(MASPreconditioner.cu:376-481: banks of 32 consecutive items, bank-local
connected components numbered by lowest lane, globally by bank order), both
on the library's partition: the same number of levels, the same item count
per level and the same item of every block row at every level."""
import numpy as np
import pytest
import scipy.sparse as sp

import lss
from lss import gen
from oracle import oracle as O


def _permuted_bsr(A, bd, perm):
    nb = A.shape[0] // bd
    # scalar permutation from the block permutation (old block -> new block)
    inv = np.empty(nb, np.int64)
    inv[perm] = np.arange(nb)
    p = (inv[:, None] * bd + np.arange(bd)[None, :]).ravel()  # new scalar -> old scalar
    Ar = sp.csr_matrix((A.data, A.indices, A.indptr), shape=A.shape)  # outer index = row
    Ap = Ar[p][:, p].tobsr(blocksize=(bd, bd))
    Ap.sort_indices()
    return nb, Ap.indptr.astype(np.int32), Ap.indices.astype(np.int32), Ap.data.reshape(-1)


def _cases():
    return [
        pytest.param(lambda: gen.workload_elasticity_inclusion(seed=0, nodes=16)[0], 3, id="elasticity_16"),
        pytest.param(lambda: gen.workload_elasticity_lognormal(seed=1, nodes=14)[0], 3, id="springs_14"),
        pytest.param(lambda: gen.workload_delaunay_laplacian(seed=0, npts=40_000)[0], 1, id="delaunay_40k"),
    ]


@pytest.mark.parametrize("make,bd", _cases())
def test_coarse_space_matches_oracle(make, bd, built):
    A = make().tocsc()
    A.sum_duplicates()
    perm, offs = lss.partition_pattern(A, bd)
    items, cmaps = lss.coarse_space(A, bd, 4)
    nb, rows, cols, vals = _permuted_bsr(A, bd, perm)
    m = O.Mas(nb, bd, rows, cols, vals, offs, max_coarse_levels=4)
    assert m.status == 0
    assert m.levels() == len(items), (m.levels(), items)
    for l in range(len(items)):
        assert m.level_items(l) == items[l], (l, m.level_items(l), items[l])
    for l in range(1, len(items)):
        np.testing.assert_array_equal(m.coarse_map(l), cmaps[l - 1])
    # the levels shrink: bank-aligned connected parts give roughly 32x per level
    assert all(items[l + 1] < items[l] for l in range(len(items) - 1))
