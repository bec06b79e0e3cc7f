"""Synthetic workload generators: shapes, symmetry, definiteness (CPU)."""
import numpy as np
import scipy.sparse as sp

from conftest import built  # noqa: F401


def test_elasticity_small_workload_shape(built):
    from lss import gen
    A, b, info = gen.workload_elasticity_inclusion(seed=0, nodes=20)
    assert A.shape == (24000, 24000)
    assert abs(A - A.T).max() <= 1e-9 * abs(A).max()
    # 15-point block stencil of the Kuhn split (about 1.0M scalar slots), with
    # the exact zeros of axis-aligned couplings and clamped rows pruned
    assert 0.7e6 < A.nnz < 1.1e6
    assert len(b) == 24000
    d = A.diagonal()
    assert d.min() > 0 and d.max() / d.min() > 1e4  # stiff inclusion present


def test_elasticity_is_spd(built):
    from lss import gen
    A, _, _ = gen.workload_elasticity_inclusion(seed=2, nodes=5)
    w = np.linalg.eigvalsh(A.toarray())
    assert w.min() > 0


def test_elasticity_springs_and_clamp(built):
    from lss import gen
    rng = np.random.default_rng(0)
    E = rng.lognormal(size=6 * 3 ** 3)
    A = gen.elasticity_cube(4, 4, 4, E, spring_nodes=[60], spring_k=1e8)
    assert A[180, 180] > 1e8 and A[0, 0] == 1.0 and A[0, 1] == 0.0


def test_delaunay_laplacian(built):
    from lss import gen
    A, b, info = gen.workload_delaunay_laplacian(seed=0, npts=800)
    assert A.shape == (800, 800)
    assert abs(A - A.T).max() <= 1e-9 * abs(A).max()
    assert info["collapsed"] > 0
    assert np.linalg.eigvalsh(A.toarray()).min() > 0
    d = A.diagonal()
    assert d.max() / np.median(d) > 100  # collapsed triangles make stiff rows
