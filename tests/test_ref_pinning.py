"""Parity pinning: the oracle against the REFERENCE'S OWN selection code (CPU).

tests/golden/ref_selection.npz was written by tests/golden/make_ref_golden.py
from GPUHybrid::select_bad_dofs, filter_subdomains,
expand_subdomains_to_strongly_connected and
decompose_subdomains_to_disjoint_subsets (GPUHybrid.cu:691-991), compiled from
the reference sources on the host (oracle/build_ref.py).  The C and numpy
restatements must reproduce it exactly: the GMM selection, the final stiff
set, the subdomains, and the GMM statistics bit for bit.  The fixtures the GPU
tests compare against (selection_golden.npz) must equal it too, so the GPU's
index sets are pinned to the reference's code through them.  Where the
reference build itself is available (oracle/_ref), it is also run live on
further seeded systems."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_npz_matrix, reference_matrices
from oracle import oracle as O

REF = dict(np.load(os.path.join(GOLDEN, "ref_selection.npz")))
META = json.load(open(os.path.join(GOLDEN, "ref_selection.json")))
PARAM_SETS = json.load(open(os.path.join(GOLDEN, "selection_golden.json")))["param_sets"]
STAT_KEYS = ("global_mean", "global_var", "mean0", "mean1", "var0", "var1", "gmm_iters")


def _canonical(subs):
    subs = [np.sort(np.asarray(s, np.int32)) for s in subs if len(s)]
    subs.sort(key=lambda s: int(s[0]))
    return subs


def _synthetic(kind, kw):
    from lss import gen
    A, _, _ = getattr(gen, "workload_" + kind)(**kw)
    A = A.tocsc()
    A.sum_duplicates()
    return A


def _cases():
    out = []
    for key, m in sorted(META["cases"].items()):
        if "/" in key:
            name, pname = key.split("/")
            out.append(pytest.param(key, ("matrix", name), m["params"], id=key))
        else:
            kind, kw = META["synthetic"][key]
            out.append(pytest.param(key, ("synthetic", kind, kw), m["params"], id=key))
    return out


def _matrix(src):
    if src[0] == "matrix":
        mats = reference_matrices()
        if src[1] not in mats:
            pytest.skip(f"{src[1]} not generated here (tests/golden/make_golden.py)")
        return load_npz_matrix(mats[src[1]])
    return _synthetic(src[1], src[2])


def _check(key, A, params, pipeline):
    allsel, subs = pipeline(A, params)[:2]
    subs = _canonical(subs)
    np.testing.assert_array_equal(allsel, REF[key + "/selected"])
    np.testing.assert_array_equal(np.cumsum([0] + [len(s) for s in subs]), REF[key + "/sub_offsets"])
    got = np.concatenate(subs) if subs else np.zeros(0, np.int32)
    np.testing.assert_array_equal(got, REF[key + "/sub_dofs"])


@pytest.mark.parametrize("key,src,params", _cases())
def test_c_oracle_reproduces_reference_build(key, src, params):
    A = _matrix(src)
    p = dict(O.DEFAULTS)
    p.update(params)
    sel, st = O.c_gmm_select(O.c_row_l1_norms(A), p["gmm_jump_threshold"], p["gmm_tol"], p["max_gmm_iterations"])
    np.testing.assert_array_equal(sel, REF[key + "/gmm_selection"])
    ref_stats = REF[key + "/gmm_stats"]
    got = np.array([st[k] for k in STAT_KEYS], dtype=np.float64)
    # the sequential host reductions of both sides round alike: bit for bit
    np.testing.assert_array_equal(got, ref_stats)
    _check(key, A, params, O.c_select_pipeline)


@pytest.mark.parametrize("key,src,params", _cases())
def test_numpy_oracle_reproduces_reference_build(key, src, params):
    A = _matrix(src)
    _check(key, A, params, O.np_select_pipeline)


@pytest.mark.parametrize("name", sorted(reference_matrices()))
@pytest.mark.parametrize("pname", sorted(PARAM_SETS))
def test_gpu_fixtures_equal_reference_build(name, pname, golden):
    """The fixtures of the GPU parity tests are the reference build's outputs."""
    key = f"{name}/{pname}"
    for part in ("gmm_selection", "selected", "sub_offsets"):
        np.testing.assert_array_equal(golden[f"{key}/{part}"], REF[f"{key}/{part}"])


def _live():
    if O.ref_lib() is None:
        pytest.skip("the reference build (oracle/_ref) needs a reference checkout")


@pytest.mark.parametrize("seed", [3, 4, 5])
@pytest.mark.parametrize("case", ["inclusion", "springs", "delaunay"])
def test_reference_build_live_against_oracle(case, seed):
    """Further seeded systems (not in the fixtures), every parameter set: the
    reference's code and the C oracle give identical selections and stats."""
    _live()
    if case == "inclusion":
        A = _synthetic("elasticity_inclusion", {"seed": seed, "nodes": 14, "radius": 0.2 + 0.03 * seed})
    elif case == "springs":
        A = _synthetic("elasticity_lognormal", {"seed": seed, "nodes": 12})
    else:
        A = _synthetic("delaunay_laplacian", {"seed": seed, "npts": 20_000})
    for pname, params in PARAM_SETS.items():
        raw, subs, stats = O.ref_select_pipeline(A, params)
        p = dict(O.DEFAULTS)
        p.update(params)
        sel, st = O.c_gmm_select(O.c_row_l1_norms(A), p["gmm_jump_threshold"], p["gmm_tol"],
                                 p["max_gmm_iterations"])
        np.testing.assert_array_equal(sel, raw)
        for k in STAT_KEYS:
            assert st[k] == stats[k], (pname, k, st[k], stats[k])
        allc, subc, _ = O.c_select_pipeline(A, params)
        subs = _canonical(subs)
        allr = np.sort(np.concatenate(subs)) if subs else np.zeros(0, np.int32)
        np.testing.assert_array_equal(allc, allr)
        assert [s.tolist() for s in _canonical(subc)] == [s.tolist() for s in subs]


def test_reference_build_edge_cases():
    """Edge cases the reference code handles: no jump (nothing selected),
    zero GMM iterations, and a 1x1 system."""
    _live()
    import scipy.sparse as sp
    A = sp.diags([np.full(99, -1.0), np.full(100, 4.0), np.full(99, -1.0)], [-1, 0, 1], format="csc")
    A = (A + sp.diags(np.linspace(0, 0.5, 100))).tocsc()
    for params in ({}, {"max_gmm_iterations": 0}, {"gmm_jump_threshold": 1.0001}):
        raw, subs, _ = O.ref_select_pipeline(A, params)
        allc, subc, _ = O.c_select_pipeline(A, params)
        allr = np.sort(np.concatenate(subs)) if subs else np.zeros(0, np.int32)
        np.testing.assert_array_equal(allc, allr)
    one = sp.csc_matrix(np.array([[5.0]]))
    raw, subs, _ = O.ref_select_pipeline(one, {})
    allc, _, _ = O.c_select_pipeline(one, {})
    assert len(raw) == 0 or np.array_equal(np.sort(raw), allc)


@pytest.mark.parametrize("key,src,params", _cases())
def test_product_postprocessing_reproduces_reference_build(key, src, params, built):
    """The library's own host post-processing (lss_postprocess_selection: the
    filter with the selected submatrix's Gershgorin sums, the one-ring
    expansion and the decomposition, as HybridSolver::select_stiff runs them)
    fed with the reference build's GMM selection gives the reference build's
    final stiff set and subdomains exactly."""
    import lss
    A = _matrix(src)
    subs = _canonical(lss.postprocess_selection(A, params, REF[key + "/gmm_selection"]))
    allsel = np.sort(np.concatenate(subs)) if subs else np.zeros(0, np.int32)
    np.testing.assert_array_equal(allsel, REF[key + "/selected"])
    if not params.get("decompose_subdomains", True):
        # The reference factors one block holding every selected DOF; the
        # library factors its connected components (the same operator, the
        # inverse being block diagonal over them): the components partition the
        # reference's block and no entry of A couples two of them.
        assert len(REF[key + "/sub_offsets"]) == 2
        comp = np.full(A.shape[0], -1)
        for q, c in enumerate(subs):
            comp[c] = q
        Ac = A.tocsc()
        for q, c in enumerate(subs):
            for k in c:
                rows = Ac.indices[Ac.indptr[k]:Ac.indptr[k + 1]]
                other = comp[rows]
                assert np.all((other == -1) | (other == q)), (key, k)
        return
    np.testing.assert_array_equal(np.cumsum([0] + [len(s) for s in subs]), REF[key + "/sub_offsets"])
    got = np.concatenate(subs) if subs else np.zeros(0, np.int32)
    np.testing.assert_array_equal(got, REF[key + "/sub_dofs"])
