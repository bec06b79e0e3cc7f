"""The oracle against the golden fixtures and the reference's documented
semantics (CPU only).  Two restatements -- C (oracle/lss_oracle.c) and numpy
(oracle/oracle.py) -- must agree with each other and with the committed
golden selections of the reference's example matrices."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import GOLDEN, load_npz_matrix, reference_matrices
from oracle import oracle as O

PARAM_SETS = json.load(open(os.path.join(GOLDEN, "selection_golden.json")))["param_sets"]


@pytest.mark.parametrize("name", sorted(reference_matrices()))
@pytest.mark.parametrize("pname", sorted(PARAM_SETS))
def test_selection_matches_golden(name, pname, golden):
    A = load_npz_matrix(reference_matrices()[name])
    params = PARAM_SETS[pname]
    rn = O.c_row_l1_norms(A)
    assert rn.sum() == pytest.approx(golden[f"{name}/rn_sum"][0], rel=1e-14)
    p = dict(O.DEFAULTS)
    p.update(params)
    sel, stats = O.c_gmm_select(rn, p["gmm_jump_threshold"], p["gmm_tol"], p["max_gmm_iterations"])
    np.testing.assert_array_equal(sel, golden[f"{name}/{pname}/gmm_selection"])
    allsel, subs, _ = O.c_select_pipeline(A, params)
    np.testing.assert_array_equal(allsel, golden[f"{name}/{pname}/selected"])
    offs = np.cumsum([0] + [len(s) for s in subs])
    np.testing.assert_array_equal(offs, golden[f"{name}/{pname}/sub_offsets"])
    allnp, subsnp = O.np_select_pipeline(A, params)
    np.testing.assert_array_equal(allnp, allsel)


def _bimodal_rows(n=400, stiff=(10, 20), seed=1):
    """Tridiagonal SPD matrix with a block of stiff rows."""
    rng = np.random.default_rng(seed)
    d = 2.0 + rng.uniform(0, 0.1, n)
    scale = np.ones(n)
    scale[stiff[0]:stiff[1]] = 1e6
    main = d * scale
    off = -0.5 * np.sqrt(scale[:-1] * scale[1:])
    return sp.diags([off, main, off], [-1, 0, 1], format="csc")


def test_gmm_selects_stiff_block():
    A = _bimodal_rows()
    sel, st = O.c_gmm_select(O.c_row_l1_norms(A), 10.0, 1e-3, 20)
    assert set(sel.tolist()) == set(range(10, 20))
    assert st["jump_passed"] == 1
    sel2, _ = O.np_gmm_select(O.np_row_l1_norms(A), 10.0, 1e-3, 20)
    np.testing.assert_array_equal(sel, sel2)


def test_gmm_no_jump_selects_nothing():
    A = sp.diags([np.full(99, -1.0), np.full(100, 4.0), np.full(99, -1.0)], [-1, 0, 1], format="csc")
    A = A + sp.diags(np.linspace(0, 0.5, 100))
    sel, st = O.c_gmm_select(O.c_row_l1_norms(A), 100.0, 1e-3, 20)
    assert len(sel) == 0 and st["jump_passed"] == 0


def test_gmm_zero_iterations_selects_nothing():
    # thrust device_vector gammas start at 0 (GPUHybrid.cu:787-790): g0 < g1 never holds
    A = _bimodal_rows()
    sel, st = O.c_gmm_select(O.c_row_l1_norms(A), 10.0, 1e-3, 0)
    assert len(sel) == 0 and st["estep_count"] == 0
    sel2, _ = O.np_gmm_select(O.np_row_l1_norms(A), 10.0, 1e-3, 0)
    assert len(sel2) == 0


def test_filter_expand_decompose_semantics():
    # two stiff islands of sizes 10 and 3 in a path graph
    n = 200
    scale = np.ones(n)
    scale[20:30] = 1e6
    scale[100:103] = 1e6
    main = 2.0 * scale
    off = -0.5 * np.sqrt(scale[:-1] * scale[1:])
    A = sp.diags([off, main, off], [-1, 0, 1], format="csc")
    sel, _ = O.c_gmm_select(O.c_row_l1_norms(A), 10.0, 1e-3, 20)
    assert set(sel.tolist()) == set(range(20, 30)) | set(range(100, 103))
    # min size drops the 3-island (GPUHybrid.cu:925-929)
    kept, cnt = O.c_filter(A, sel, min_size=4, max_size=10**7, cond=1.0)
    assert set(kept.tolist()) == set(range(20, 30)) and cnt[0] == 1
    # max size drops the 10-island
    kept, cnt = O.c_filter(A, sel, min_size=1, max_size=5, cond=1.0)
    assert set(kept.tolist()) == set(range(100, 103)) and cnt[1] == 1
    # a well-conditioned island is dropped by the Gershgorin test (lmax/lmin <= 100)
    kept, cnt = O.c_filter(A, sel, min_size=1, max_size=10**7, cond=100.0)
    assert len(kept) == 0 and cnt[2] == 2
    # one-ring expansion
    ex = O.c_expand(A, np.array([50], np.int32))
    assert ex.tolist() == [49, 50, 51]
    # decomposition into components, max size
    subs = O.c_decompose(A, np.array([1, 2, 3, 10, 11], np.int32), max_size=10)
    assert [s.tolist() for s in subs] == [[1, 2, 3], [10, 11]]
    subs = O.c_decompose(A, np.array([1, 2, 3, 10, 11], np.int32), max_size=2)
    assert [s.tolist() for s in subs] == [[10, 11]]
    np_subs = O._np_components(A, np.array([1, 2, 3, 10, 11]))
    assert [s.tolist() for s in np_subs] == [[1, 2, 3], [10, 11]]


def test_oracle_method_solves_small_elasticity(built):
    from lss import gen
    A, b, _ = gen.workload_elasticity_inclusion(seed=3, nodes=8)
    s = O.CpuSolver(A, {"block_size": 3, "relative_tolerance": 1e-10, "gmm_jump_threshold": 10.0})
    assert s.status == 0
    x, info = s.solve(b)
    xd = spla.spsolve(A.tocsc(), b)
    # recurrence residual 1e-10; the true residual drifts above it on stiff systems
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1e-8
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-7
    assert s.num_stiff > 0 and info["num_iterations"] < 200


def test_oracle_mas_is_spd(built):
    from lss import gen
    A, _, _ = gen.workload_elasticity_inclusion(seed=4, nodes=6)
    s = O.CpuSolver(A, {"block_size": 3, "do_hybrid_precond": False})
    rng = np.random.default_rng(0)
    u, v = rng.standard_normal(A.shape[0]), rng.standard_normal(A.shape[0])
    Mu, Mv = s.precond(u), s.precond(v)
    assert abs(u @ Mv - v @ Mu) <= 1e-10 * abs(u @ Mv)
    assert u @ Mu > 0 and v @ Mv > 0
