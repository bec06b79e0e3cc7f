"""Golden fixtures produced by the REFERENCE'S OWN selection code.

oracle/build_ref.py compiles GPUHybrid::select_bad_dofs, filter_subdomains,
expand_subdomains_to_strongly_connected and
decompose_subdomains_to_disjoint_subsets (GPUHybrid.cu:691-991) from a
reference checkout on the host (thrust's sequential host backend).  This
script runs that build on

* the reference's example matrices A_contact and A_pq (tests/golden/) under
  three GPUHybrid parameter sets, and
* seeded synthetic systems of the benchmark families (small sizes),

and writes ref_selection.npz: per case the GMM selection, the final stiff set,
the subdomains (each ascending, ordered by first DOF -- the reference's own
order is that of an unordered_map) and the GMM statistics of its
"[bad_dof_selection]" log line.  For the full-size benchmark configurations it
writes ref_selection_full.json: counts and SHA-256 digests of the selections
(int32 little-endian, ascending), small enough to commit.

Run from the repository root with the path of a reference checkout:
    python tests/golden/make_ref_golden.py <reference checkout> [--full]
"""
import hashlib
import json
import os
import sys
import time

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "local-stiff-solver_gb300"))

from oracle import build_ref  # noqa: E402
from oracle import oracle as O  # noqa: E402

PARAM_SETS = {
    "spec_example": {"gmm_jump_threshold": 10.0, "gmm_tol": 1e-3, "max_gmm_iterations": 20,
                     "decompose_subdomains": True, "min_subdomain_size": 4, "expand_subdomains": True},
    "spec_defaults": {},
    "no_decompose": {"gmm_jump_threshold": 10.0, "decompose_subdomains": False},
}

# seeded synthetic cases: (generator call, parameter set)
SYNTHETIC = {
    "elasticity_inclusion_20": ("elasticity_inclusion", {"seed": 0, "nodes": 20},
                                {"gmm_jump_threshold": 10.0, "min_subdomain_size": 4}),
    "elasticity_inclusion_16_r03": ("elasticity_inclusion", {"seed": 2, "nodes": 16, "radius": 0.3},
                                    {"gmm_jump_threshold": 10.0, "min_subdomain_size": 4}),
    "lognormal_springs_16": ("elasticity_lognormal", {"seed": 0, "nodes": 16},
                             {"decompose_subdomains": False}),
    "delaunay_40k": ("delaunay_laplacian", {"seed": 0, "npts": 40_000},
                     {"gmm_jump_threshold": 10.0, "min_subdomain_size": 4}),
}

# full-size benchmark configurations, with the benchmark's own parameters
FULL = {
    "elasticity_24k": ("elasticity_inclusion", {"seed": 0, "nodes": 20},
                       {"gmm_jump_threshold": 10.0, "min_subdomain_size": 4}),
    "elasticity_3m": ("elasticity_lognormal", {"seed": 0, "nodes": 100}, {"decompose_subdomains": False}),
}


def synthetic(kind, kw):
    from lss import gen
    A, b, _ = getattr(gen, "workload_" + kind)(**kw)
    A = A.tocsc()
    A.sum_duplicates()
    return A


def canonical(subs):
    subs = [np.sort(np.asarray(s, np.int32)) for s in subs if len(s)]
    subs.sort(key=lambda s: int(s[0]))
    return subs


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def record(out, meta, key, A, params):
    t = time.time()
    raw, subs, stats = O.ref_select_pipeline(A, params)
    subs = canonical(subs)
    allsel = np.sort(np.concatenate(subs)) if subs else np.zeros(0, np.int32)
    out[key + "/gmm_selection"] = raw.astype(np.int32)
    out[key + "/selected"] = allsel.astype(np.int32)
    out[key + "/sub_offsets"] = np.cumsum([0] + [len(s) for s in subs]).astype(np.int32)
    out[key + "/sub_dofs"] = np.concatenate(subs).astype(np.int32) if subs else np.zeros(0, np.int32)
    out[key + "/gmm_stats"] = np.array([stats[k] for k in ("global_mean", "global_var", "mean0", "mean1",
                                                           "var0", "var1", "gmm_iters")])
    meta[key] = {"n": int(A.shape[0]), "nnz": int(A.nnz), "params": params, "gmm_selected": int(len(raw)),
                 "selected": int(len(allsel)), "subdomains": len(subs), "seconds": round(time.time() - t, 3)}
    print(key, meta[key], flush=True)


def main(reference, full):
    lib = build_ref.build(reference, force=True)
    if lib is None:
        raise SystemExit("reference checkout not found: " + reference)
    out, meta = {}, {}
    mats = {"A_contact": os.path.join(HERE, "A_contact.npz"), "A_pq": os.path.join(HERE, "_large", "A_pq.npz")}
    for name, path in mats.items():
        if not os.path.exists(path):
            raise SystemExit(f"{path} missing: run tests/golden/make_golden.py first")
        z = np.load(path)
        n = len(z["indptr"]) - 1
        A = sp.csc_matrix((z["data"], z["indices"], z["indptr"]), shape=(n, n))
        for pname, params in PARAM_SETS.items():
            record(out, meta, f"{name}/{pname}", A, params)
    for name, (kind, kw, params) in SYNTHETIC.items():
        record(out, meta, name, synthetic(kind, kw), params)
    np.savez_compressed(os.path.join(HERE, "ref_selection.npz"), **out)
    with open(os.path.join(HERE, "ref_selection.json"), "w") as f:
        json.dump({"synthetic": {k: [v[0], v[1]] for k, v in SYNTHETIC.items()}, "cases": meta}, f, indent=1,
                  sort_keys=True)
    if full:
        res = {}
        for name, (kind, kw, params) in FULL.items():
            A = synthetic(kind, kw)
            t = time.time()
            raw, subs, stats = O.ref_select_pipeline(A, params)
            subs = canonical(subs)
            allsel = np.sort(np.concatenate(subs)) if subs else np.zeros(0, np.int32)
            res[name] = {"generator": [kind, kw], "params": params, "n": int(A.shape[0]), "nnz": int(A.nnz),
                         "gmm_selected": int(len(raw)), "selected": int(len(allsel)), "subdomains": len(subs),
                         "sha256_gmm_selection": digest(raw), "sha256_selected": digest(allsel),
                         "sha256_sub_offsets": digest(np.cumsum([0] + [len(s) for s in subs])),
                         "gmm_stats": {k: stats[k] for k in ("global_mean", "global_var", "mean0", "mean1",
                                                              "var0", "var1", "gmm_iters")},
                         "seconds": round(time.time() - t, 2)}
            print(name, res[name], flush=True)
        with open(os.path.join(HERE, "ref_selection_full.json"), "w") as f:
            json.dump(res, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if len(args) != 1:
        raise SystemExit("usage: python tests/golden/make_ref_golden.py <reference checkout> [--full]")
    main(args[0], "--full" in sys.argv)
