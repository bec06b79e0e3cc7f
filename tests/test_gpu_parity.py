"""GPU parity tests: the CUDA path (through the C ABI) against the oracle.

Tolerances, stated per test:
  * stiff-DOF index sets: identical (bit-exact integer parity);
  * l1 row norms: 1e-13 relative (summation order differs);
  * SpMV: 1e-13 of |A||x| per entry;
  * MAS / hybrid preconditioner in FP64 against the oracle on the same
    partition: 1e-7 relative (the bank inverses are computed in a different
    index order; banks that straddle a 1e6 stiffness jump have condition
    numbers near 1e8, so their FP64 inverses agree to about 1e-8);
  * FP32 MAS (mixed mode) against FP64: 2e-3 relative;
  * solves: true relative residual <= max(1e-8, 20 * floor) and <= 1e-6
    relative error against scipy's FP64 sparse direct solve, where
    floor = eps * || |A| |x| || / ||b|| is the rounding floor of the residual
    itself (about 8e-8 for A_contact, whose sparse direct solution reaches
    only 2.8e-7).
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import GOLDEN, load_npz_matrix, reference_matrices

pytestmark = pytest.mark.gpu

PARAM_SETS = json.load(open(os.path.join(GOLDEN, "selection_golden.json")))["param_sets"]


def _solver(params, gb300=None):
    import lss
    p = {"solver": "GPUHybrid", "GPUHybrid": dict(params)}
    if gb300:
        p["gb300"] = gb300
    return lss.Solver.create(p)


@pytest.fixture(scope="module")
def elast20(built):
    from lss import gen
    A, b, _ = gen.workload_elasticity_inclusion(seed=0, nodes=20)
    return A.tocsc(), b


@pytest.fixture(scope="module")
def lap(built):
    from lss import gen
    A, b, _ = gen.workload_delaunay_laplacian(seed=1, npts=30000)
    return A.tocsc(), b


def test_row_l1_norms_match_oracle(built):
    import lss
    from oracle import oracle as O
    for name, path in reference_matrices().items():
        A = load_npz_matrix(path)
        g = lss.row_l1_norms(A)
        c = O.c_row_l1_norms(A)
        np.testing.assert_allclose(g, c, rtol=1e-13, atol=0)


@pytest.mark.parametrize("name", sorted(reference_matrices()))
@pytest.mark.parametrize("pname", sorted(PARAM_SETS))
def test_selection_matches_golden(name, pname, golden):
    A = load_npz_matrix(reference_matrices()[name])
    s = _solver(dict(PARAM_SETS[pname], block_size=1))
    s.factorize(A)
    np.testing.assert_array_equal(s.gmm_selection(), golden[f"{name}/{pname}/gmm_selection"])
    np.testing.assert_array_equal(s.selected_dofs(), golden[f"{name}/{pname}/selected"])
    if PARAM_SETS[pname].get("decompose_subdomains", True):
        offs = np.cumsum([0] + [len(x) for x in s.subdomains()])
        np.testing.assert_array_equal(offs, golden[f"{name}/{pname}/sub_offsets"])
    assert s.name() == "GPUHybrid"


@pytest.mark.parametrize("case", ["elasticity", "laplacian", "lognormal_springs"])
def test_selection_matches_oracle_on_workloads(case, built):
    from lss import gen
    from oracle import oracle as O
    if case == "elasticity":
        A, _, _ = gen.workload_elasticity_inclusion(seed=5, nodes=14, E_ratio=1e5)
        params = {"block_size": 3, "gmm_jump_threshold": 10.0, "min_subdomain_size": 4}
    elif case == "laplacian":
        A, _, _ = gen.workload_delaunay_laplacian(seed=2, npts=40000)
        params = {"block_size": 1, "gmm_jump_threshold": 10.0, "min_subdomain_size": 4}
    else:
        A, _, _ = gen.workload_elasticity_lognormal(seed=1, nodes=16)
        params = {"block_size": 3, "gmm_jump_threshold": 10.0}
    A = A.tocsc()
    s = _solver(params)
    s.factorize(A)
    ref_all, ref_subs, _ = O.c_select_pipeline(A, params)
    np.testing.assert_array_equal(s.selected_dofs(), ref_all)
    got = s.subdomains()
    assert len(got) == len(ref_subs)
    for a, b in zip(got, ref_subs):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("lanes", [0, 1, 2, 4, 8, 16, 32])
@pytest.mark.parametrize("bs", [1, 3])
def test_spmv_matches_scipy(bs, lanes, elast20, lap):
    """Every launch shape (threads per block row; 0 = autotuned), including
    groups narrower than the block size, where one thread stores several
    components of the block row."""
    A = elast20[0] if bs == 3 else lap[0]
    s = _solver({"block_size": bs, "do_hybrid_precond": False}, {"spmv_lanes": lanes} if lanes else None)
    s.factorize(A)
    if lanes:
        assert s.get_info()["spmv_lanes"] == lanes
    x = np.random.default_rng(0).standard_normal(A.shape[0])
    y = s.spmv(x)
    ref = A.tocsr() @ x  # outer index = row, like the reference (the matrix is symmetric)
    bound = abs(A.tocsr()) @ abs(x)
    assert np.all(np.abs(y - ref) <= 1e-13 * bound + 1e-300)


@pytest.mark.parametrize("lanes", [1, 2, 4, 16])
@pytest.mark.parametrize("outer", ["fp64", "df32"])
@pytest.mark.parametrize("bs", [1, 3])
def test_outer_spmv_matches_scipy(bs, outer, lanes, elast20, lap):
    """The PCG's own A p: FP64, or double-float on the FP32 pipe (values and
    p split into FP32 high and low words, error-free products and sums).  Both
    within 1e-13 of |A||x| per entry; the double-float form carries about
    2^-47 relative error per term, FP64 about 2^-53."""
    A = elast20[0] if bs == 3 else lap[0]
    s = _solver({"block_size": bs, "do_hybrid_precond": False}, {"outer_spmv": outer, "spmv_lanes": lanes})
    s.factorize(A)
    assert s.get_info()["outer_spmv"] == outer
    x = np.random.default_rng(3).standard_normal(A.shape[0]) * np.exp(np.random.default_rng(4).standard_normal(A.shape[0]))
    y = s.spmv_outer(x)
    ref = A.tocsr() @ x
    bound = abs(A.tocsr()) @ abs(x)
    assert np.all(np.abs(y - ref) <= 1e-13 * bound + 1e-300)


def _oracle_with_product_partition(A, s, params, **kw):
    from oracle import oracle as O
    perm, offs = s.partition()
    return O.CpuSolver(A, params, perm=perm, part_offsets=offs, **kw)


@pytest.mark.parametrize("bs", [1, 3])
def test_mas_apply_matches_oracle(bs, elast20, lap):
    A = elast20[0] if bs == 3 else lap[0]
    params = {"block_size": bs, "do_hybrid_precond": False}
    s = _solver(params)
    s.factorize(A)
    o = _oracle_with_product_partition(A, s, params)
    info = s.get_info()
    r = np.random.default_rng(1).standard_normal(A.shape[0])
    z = s.mas_apply(r)
    zo = o.precond(r)
    err = np.linalg.norm(z - zo) / np.linalg.norm(zo)
    assert err < 1e-7, (err, info["mas_levels"])
    # FP32 storage of the inverses (mixed precision mode)
    s32 = _solver(params, {"precision": "mixed"})
    s32.factorize(A)
    z32 = s32.mas_apply(r)
    assert np.linalg.norm(z32 - zo) / np.linalg.norm(zo) < 2e-3


def test_hybrid_precond_matches_oracle(elast20):
    A = elast20[0]
    params = {"block_size": 3, "gmm_jump_threshold": 10.0, "min_subdomain_size": 4}
    s = _solver(params)
    s.factorize(A)
    omega = s.get_info()["mas_omega"]
    o = _oracle_with_product_partition(A, s, params, mas_omega=omega)
    assert o.num_stiff == len(s.selected_dofs()) > 0
    r = np.random.default_rng(2).standard_normal(A.shape[0])
    z = s.precond(r)
    zo = o.precond(r)
    assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 1e-7
    # the automatic damping agrees with the oracle's own estimate
    o2 = _oracle_with_product_partition(A, s, params)
    assert abs(o2.omega - omega) / omega < 1e-6
    # additive composition (MASSolver.cu:583-615)
    sa = _solver(params, {"composition": "additive"})
    sa.factorize(A)
    oa = _oracle_with_product_partition(A, sa, params, additive=True)
    za, zoa = sa.precond(r), oa.precond(r)
    assert np.linalg.norm(za - zoa) / np.linalg.norm(zoa) < 1e-7


@pytest.fixture(scope="module")
def springs16(built):
    from lss import gen
    A, b, _ = gen.workload_elasticity_lognormal(seed=0, nodes=16)
    return A.tocsc(), b


@pytest.mark.parametrize("lanes", [1, 2, 4])
def test_mixed_precond_every_residual_shape(lanes, springs16):
    """Mixed mode: the FP32 residual SpMV inside the multiplicative
    composition at each launch shape; FP32 MAS against the FP64 oracle with the
    same damping: 2e-3 relative.  (The FP32 copy of A rounds every term of
    r - A z, so rows whose terms cancel from a much larger scale -- the rim of
    a 1e6 inclusion -- carry errors of 6e-8 times that scale; the lognormal
    moduli with diagonal penalty springs have no such rows.)"""
    A = springs16[0]
    params = {"block_size": 3, "decompose_subdomains": False}
    s = _solver(params, {"precision": "mixed", "spmv_lanes": lanes})
    s.factorize(A)
    info = s.get_info()
    assert info["spmv_lanes"] == info["spmv_lanes_fp32"] == lanes
    assert len(s.selected_dofs()) > 0  # the composition runs its residual SpMV
    o = _oracle_with_product_partition(A, s, params, mas_omega=info["mas_omega"])
    r = np.random.default_rng(2).standard_normal(A.shape[0])
    z, zo = s.precond(r), o.precond(r)
    assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 2e-3


def test_mas_bf16_offdiagonal_tiles(springs16):
    """Mixed precision with the level-0 off-diagonal inverse tiles in BF16:
    the MAS apply stays within 2e-2 of the FP32-tile one (BF16 keeps 8 bits),
    the solve converges to the parity bar, and the level-0 inverse bytes drop
    by a third."""
    A, b = springs16
    params = {"block_size": 3, "relative_tolerance": 1e-8, "decompose_subdomains": False}
    s32 = _solver(params, {"precision": "mixed"})
    s16 = _solver(params, {"precision": "mixed", "mas_offdiag": "bf16"})
    s32.factorize(A)
    s16.factorize(A)
    r = np.random.default_rng(9).standard_normal(A.shape[0])
    z32, z16 = s32.mas_apply(r), s16.mas_apply(r)
    assert np.linalg.norm(z16 - z32) / np.linalg.norm(z32) < 2e-2
    i32, i16 = s32.get_info(), s16.get_info()
    assert i16["mas_inverse_bytes"] < 0.8 * i32["mas_inverse_bytes"]
    x = s16.solve(b)
    _check_solution(A, b, x)
    assert s16.get_info()["status"] == "converged_rel"


def test_mixed_matches_fp64_on_penalty_springs(built):
    """Lognormal moduli and 1e8 diagonal penalty springs: the mixed mode
    converges like the FP64 mode (same damping estimate within 1e-4, at most
    10% more iterations) at every launch shape of the FP32 residual."""
    from lss import gen
    A, b, _ = gen.workload_elasticity_lognormal(seed=0, nodes=24)
    A = A.tocsc()
    params = {"block_size": 3, "relative_tolerance": 1e-8, "decompose_subdomains": False}
    ref = _solver(params)
    ref.factorize(A)
    ref.solve(b)
    i64 = ref.get_info()
    assert i64["status"] == "converged_rel"
    for lanes in [1, 2, 4]:
        s = _solver(params, {"precision": "mixed", "spmv_lanes": lanes})
        s.factorize(A)
        x = s.solve(b)
        inf = s.get_info()
        assert inf["status"] == "converged_rel", (lanes, inf["status"])
        assert abs(inf["mas_lambda_max"] - i64["mas_lambda_max"]) <= 1e-4 * i64["mas_lambda_max"]
        assert inf["num_iterations"] <= 1.1 * i64["num_iterations"] + 2, (lanes, inf["num_iterations"])
        _check_solution(A, b, x)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_mixed_high_contrast_reaches_tolerance(seed, built):
    """E ratio 1e7: the double-float outer product's 2^-48 per term can set a
    residual floor above 1e-8 here; the refinement restarts then run with the
    FP64 product, so the returned x meets max(1e-8, 2 x the FP64 floor) and
    1e-6 of scipy's sparse direct solve.  (Seed 2's FP64 floor
    eps || |A| |x| || / ||b|| is 3.9e-8: scipy's direct solve itself stops at
    2.9e-8.)"""
    from lss import gen
    A, b, _ = gen.workload_elasticity_inclusion(seed=seed, nodes=20, E_ratio=1e7)
    A = A.tocsc()
    s = _solver({"block_size": 3, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0,
                 "min_subdomain_size": 4}, {"precision": "mixed"})
    s.factorize(A)
    x = s.solve(b)
    Ar = _outer_as_row(A)
    floor = np.finfo(np.float64).eps * np.linalg.norm(abs(Ar) @ abs(x)) / np.linalg.norm(b)
    rel = np.linalg.norm(b - Ar @ x) / np.linalg.norm(b)
    assert rel <= max(1e-8, 2 * floor), (rel, floor, s.get_info()["refinements"])
    xd = spla.spsolve(Ar.tocsc(), b)
    assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_large_stiff_subdomain(precision, built):
    """A 0.3-radius x1e6 inclusion on a 16^3-node cube makes one stiff
    subdomain of 3,168 DOFs: the FP64 multifrontal factor (nested dissection,
    blocks above 160 DOFs).  The preconditioner matches the oracle's (exact
    Cholesky of the same block, same partition and damping) to 1e-7 in FP64:
    the block's condition number is 6.6e7 (cond * eps = 1.5e-8; two FP64
    direct solvers, Cholesky and SuperLU, already differ by 2.5e-10 on it),
    and the composition multiplies the stiff solve's error by A before the
    second MAS pass.  The solve reaches the parity bar."""
    from lss import gen
    A, b, _ = gen.workload_elasticity_inclusion(seed=2, nodes=16, radius=0.3)
    A = A.tocsc()
    params = {"block_size": 3, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0, "min_subdomain_size": 4}
    s = _solver(params, {"precision": precision})
    s.factorize(A)
    info = s.get_info()
    assert info["max_subdomain_dofs"] > 1000, info["max_subdomain_dofs"]
    assert info["multifrontal_subdomains"] == 1 and info["multifrontal_levels"] > 3, info
    if precision == "fp64":
        o = _oracle_with_product_partition(A, s, params, mas_omega=info["mas_omega"])
        r = np.random.default_rng(5).standard_normal(A.shape[0])
        z, zo = s.precond(r), o.precond(r)
        assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 1e-7
    x = s.solve(b)
    _check_solution(A, b, x)
    assert s.get_info()["status"] == "converged_rel"


def test_multifrontal_matches_sparse_lu(built):
    """The stiff-block solve alone, on a 14k-DOF subdomain (0.35-radius x1e6
    inclusion in a 30^3-node cube): with the additive composition,
    precond(r) - mas(r) is exactly A_SS^-1 r_S on the stiff DOFs and zero
    elsewhere.  Compared with scipy's sparse LU of every stiff block to 1e-9
    (FP64 throughout; the blocks' condition numbers near 1e8 put two FP64
    direct solvers about 1e-10 apart), twice (the factor and the solve are
    deterministic)."""
    import scipy.sparse.linalg as spla
    from lss import gen
    A, _, _ = gen.workload_elasticity_inclusion(seed=3, nodes=30, radius=0.35)
    A = A.tocsc()
    params = {"block_size": 3, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0, "min_subdomain_size": 4}
    s = _solver(params, {"composition": "additive"})
    s.factorize(A)
    info = s.get_info()
    assert info["max_subdomain_dofs"] > 10000, info["max_subdomain_dofs"]
    r = np.random.default_rng(9).standard_normal(A.shape[0])
    d = s.precond(r) - s.mas_apply(r)
    Ar = _outer_as_row(A).tocsc()
    covered = np.zeros(A.shape[0], bool)
    for sub in s.subdomains():
        sub = np.asarray(sub)
        covered[sub] = True
        x = spla.splu(Ar[sub][:, sub].tocsc()).solve(r[sub])
        assert np.linalg.norm(d[sub] - x) <= 1e-9 * np.linalg.norm(x), len(sub)
    assert np.all(d[~covered] == 0.0)
    np.testing.assert_array_equal(s.precond(r) - s.mas_apply(r), d)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_several_large_stiff_subdomains(precision, built):
    """A 120,000-point Delaunay Laplacian with 2% collapsed triangles gives
    563 stiff subdomains, 8 of them above 160 DOFs (the largest 666): they
    share one multifrontal factor, level by level.  The preconditioner
    matches the oracle's to 1e-10 in FP64, a second factorization reproduces
    it bit for bit (every sum of the factorization runs in a fixed order),
    and the solve reaches the parity bar."""
    from lss import gen
    from oracle import oracle as O
    A, b, _ = gen.workload_delaunay_laplacian(seed=1, npts=120_000)
    A = A.tocsc()
    params = {"block_size": 1, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0, "min_subdomain_size": 4}
    _, subs, _ = O.c_select_pipeline(A, params)
    assert sum(len(q) > 160 for q in subs) >= 4
    s = _solver(params, {"precision": precision})
    s.factorize(A)
    info = s.get_info()
    assert info["max_subdomain_dofs"] > 160, info["max_subdomain_dofs"]
    r = np.random.default_rng(5).standard_normal(A.shape[0])
    z = s.precond(r)
    if precision == "fp64":
        o = _oracle_with_product_partition(A, s, params, mas_omega=info["mas_omega"])
        zo = o.precond(r)
        assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 1e-10
    s.factorize(A)
    z2 = s.precond(r)
    np.testing.assert_array_equal(z2, z)
    x = s.solve(b)
    _check_solution(A, b, x)
    assert s.get_info()["status"] == "converged_rel"


@pytest.mark.parametrize("strategy", ["elbow", "kmean", "gmm"])
def test_mas_bad_dof_strategies(strategy, elast20):
    """MASSolver's bad-DOF selections in place of GPUHybrid's: the device
    scores equal numpy's on the permuted rows (|diagonal| and max
    |off-diagonal| exactly, the l1 norm to 1e-13), the selection equals the C
    oracle's on those scores (mapped back through the partition), and the
    solve reaches the parity bar."""
    from oracle import oracle as O
    A = elast20[0]
    b = elast20[1]
    gb = {"bad_dof_strategy": strategy, "bad_dof_max_block": 3000}
    params = {"block_size": 3, "relative_tolerance": 1e-8}
    s = _solver(params, gb)
    s.factorize(A)
    d, o, l1 = s.row_scores()
    perm, _ = s.partition()
    n, bd = A.shape[0], 3
    Ar = _outer_as_row(A)
    absA = abs(Ar).tocsr()
    dg = abs(Ar.diagonal())
    off = absA - sp.diags(dg)
    off.eliminate_zeros()
    offmax = np.asarray(off.max(axis=1).todense()).ravel()
    l1_ref = np.asarray(absA.sum(axis=1)).ravel()
    pos = perm[np.arange(n) // bd] * bd + np.arange(n) % bd
    np.testing.assert_array_equal(d[pos], dg)
    np.testing.assert_array_equal(o[pos], offmax)
    assert np.all(np.abs(l1[pos] - l1_ref) <= 1e-13 * l1_ref)
    score = {"elbow": d, "kmean": o, "gmm": l1}[strategy]
    args = {"elbow": (0.0, 0.0, 0, 0), "kmean": (0.2, 10.0, 32, 128), "gmm": (10.0, 1e-3, 20, 16)}[strategy]
    sel_pos = O.c_mas_select(strategy, score, *args)
    old_of = np.empty(len(perm), np.int64)
    old_of[perm] = np.arange(len(perm))
    expect = np.sort(old_of[sel_pos // bd] * bd + sel_pos % bd)
    np.testing.assert_array_equal(s.gmm_selection(), expect)
    x = s.solve(b)
    _check_solution(A, b, x)


def _outer_as_row(A):
    """The operator the solver applies: outer index = row (GPUHybrid.cu:203-209)."""
    A = A.tocsc()
    return sp.csr_matrix((A.data, A.indices, A.indptr), shape=A.shape)


def _check_solution(A, b, x, rtol=1e-8, etol=1e-6):
    Ar = _outer_as_row(A)
    xd = spla.spsolve(Ar.tocsc(), b)
    floor = np.finfo(np.float64).eps * np.linalg.norm(abs(Ar) @ abs(xd)) / np.linalg.norm(b)
    rel = np.linalg.norm(b - Ar @ x) / np.linalg.norm(b)
    assert rel <= max(rtol, 20 * floor), (rel, floor)
    err = np.linalg.norm(x - xd) / np.linalg.norm(xd)
    assert err <= etol, err
    return rel, err


@pytest.mark.parametrize("precision,outer", [("fp64", "auto"), ("mixed", "auto"), ("fp64", "df32"),
                                             ("mixed", "fp64")])
def test_solve_elasticity_inclusion(precision, outer, elast20):
    A, b = elast20
    s = _solver({"block_size": 3, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0,
                 "min_subdomain_size": 4}, {"precision": precision, "outer_spmv": outer})
    s.factorize(A)
    x = s.solve(b)
    _check_solution(A, b, x)
    info = s.get_info()
    assert info["status"] == "converged_rel" and info["num_iterations"] > 0
    assert info["num_stiff_dofs"] > 0 and info["precision"] == precision
    expect = {"auto": "df32" if precision == "mixed" else "fp64"}.get(outer, outer)  # block_size 3
    assert info["outer_spmv"] == expect


def test_solve_reference_matrices(built):
    for name, path in reference_matrices().items():
        A = load_npz_matrix(path)
        bs = 3 if name == "A_contact" else 1
        b = np.random.default_rng(0).uniform(-1, 1, A.shape[0])
        s = _solver({"block_size": bs, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0,
                     "min_subdomain_size": 4, "max_iter": 20000})
        s.factorize(A)
        x = s.solve(b)
        _check_solution(A, b, x)


def test_solve_laplacian_and_compositions(lap):
    A, b = lap
    for comp in ("multiplicative", "additive"):
        s = _solver({"block_size": 1, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0},
                    {"composition": comp})
        s.factorize(A)
        x = s.solve(b)
        _check_solution(A, b, x)


def test_initial_guess_and_zero_rhs(elast20):
    A, b = elast20
    s = _solver({"block_size": 3, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0})
    s.factorize(A)
    x = s.solve(b)
    it_cold = s.get_info()["num_iterations"]
    x2 = s.solve(b, x.copy())  # GPUHybrid uses x as the initial guess (GPUHybrid.cu:347)
    assert s.get_info()["num_iterations"] < it_cold
    z = s.solve(np.zeros_like(b), np.ones_like(b))  # GPUHybrid.cu:1433-1439
    assert np.all(z == 0) and s.get_info()["num_iterations"] == 0
    assert np.linalg.norm(x2 - x) / np.linalg.norm(x) < 1e-6


def test_max_iter_and_breakdown_status(elast20):
    A, b = elast20
    s = _solver({"block_size": 3, "relative_tolerance": 1e-14, "max_iter": 5, "gmm_jump_threshold": 10.0})
    s.factorize(A)
    s.solve(b)
    info = s.get_info()
    assert info["status"] == "max_iterations" and info["num_iterations"] == 5


def test_problematic_dofs_and_plain_modes(elast20):
    A, b = elast20
    import lss
    s = _solver({"block_size": 3, "relative_tolerance": 1e-8, "select_bad_dofs_from_l1_norm": False})
    ref = _solver({"block_size": 3, "gmm_jump_threshold": 10.0})
    ref.factorize(A)
    s.set_problematic_dofs(ref.gmm_selection())
    s.factorize(A)
    assert s.name() == "GPUAMGF"
    assert len(s.selected_dofs()) > 0
    _check_solution(A, b, s.solve(b))
    p = _solver({"block_size": 3, "relative_tolerance": 1e-8, "do_hybrid_precond": False})
    p.factorize(A)
    assert p.name() == "GPUAMG" and len(p.selected_dofs()) == 0
    _check_solution(A, b, p.solve(b))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_factorization_is_deterministic(precision, elast20):
    """Two factorizations of the same matrix (fresh solver, and the same
    solver again) give bit-identical preconditioners: the MAS Galerkin blocks
    of every coarse level and all grid reductions are summed in a fixed
    order, with no floating-point atomics, and the autotuned SpMV launch
    shape (which sets the row summation order) is kept per pattern for the
    process."""
    A, _ = elast20
    params = {"block_size": 3, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0}
    r = np.random.default_rng(11).standard_normal(A.shape[0])
    s1 = _solver(params, {"precision": precision})
    s1.factorize(A)
    assert s1.get_info()["mas_levels"] >= 2
    z1 = s1.precond(r)
    s1.factorize(A)
    np.testing.assert_array_equal(s1.precond(r), z1)
    s2 = _solver(params, {"precision": precision})
    s2.factorize(A)
    np.testing.assert_array_equal(s2.precond(r), z1)


def test_refactorize_same_pattern(elast20):
    A, b = elast20
    s = _solver({"block_size": 3, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0})
    s.analyze_pattern(A)
    for scale in (1.0, 2.0):
        A2 = (A * scale).tocsc()
        s.factorize(A2)
        _check_solution(A2, b, s.solve(b))


def test_error_paths(elast20):
    import lss
    A, b = elast20
    s = _solver({"block_size": 3})
    with pytest.raises(lss.LssError) as e:
        s.solve(b)
    assert e.value.status == "LSS_ERR_NOT_FACTORIZED"
    s.factorize(A)
    bad = b.copy()
    bad[3] = np.nan
    with pytest.raises(lss.LssError) as e:
        s.solve(bad)
    assert e.value.status == "LSS_ERR_NONFINITE"
    An = A.copy()
    An.data[7] = np.inf
    with pytest.raises(lss.LssError) as e:
        s.factorize(An)
    assert e.value.status == "LSS_ERR_NONFINITE"
    # n not a multiple of the block size
    with pytest.raises(lss.LssError) as e:
        _solver({"block_size": 3}).factorize(sp.eye(10, format="csc"))
    assert e.value.status == "LSS_ERR_INVALID_ARGUMENT"
    # device memory cap: the out-of-memory path without exhausting the GPU
    small = _solver({"block_size": 3}, {"memory_cap_bytes": 1 << 20})
    with pytest.raises(lss.LssError) as e:
        small.factorize(A)
    assert e.value.status == "LSS_ERR_OOM"
    lss.load().lss_set_memory_cap(0)
