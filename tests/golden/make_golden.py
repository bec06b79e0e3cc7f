"""Generate the golden fixtures of the stiff-DOF selection path.

Inputs: the reference's own example matrices (mats/A_contact.mtx,
mats/A_pq.mtx, documented in its README.md:44-45).  They are converted to
compressed numpy archives in the order Eigen stores them (column-compressed,
sorted indices): A_contact.npz is committed (0.4 MB); A_pq.npz (11 MB) is
written to tests/golden/_large/, which is git-ignored but travels with the
working tree.

Outputs (selection_golden.npz): for each matrix and parameter set, the l1
row-norm checksum, the GMM statistics, the raw GMM selection and the final
post-processed stiff set with its subdomains -- produced by the C oracle and
required to agree exactly with the independent numpy restatement.

Run from the repository root with the path of a reference checkout:
    python tests/golden/make_golden.py <reference checkout>
"""
import json
import os
import sys

import numpy as np
import scipy.io
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle as O  # noqa: E402

# GPUHybrid parameter sets: the reference's example config (spec/GPUHybrid.json)
# and the spec defaults (linear-solver-spec.json:646-747)
PARAM_SETS = {
    "spec_example": {"gmm_jump_threshold": 10.0, "gmm_tol": 1e-3, "max_gmm_iterations": 20,
                     "decompose_subdomains": True, "min_subdomain_size": 4, "expand_subdomains": True},
    "spec_defaults": {},
    "no_decompose": {"gmm_jump_threshold": 10.0, "decompose_subdomains": False},
}


def load_npz(path):
    z = np.load(path)
    n = len(z["indptr"]) - 1
    return sp.csc_matrix((z["data"], z["indices"], z["indptr"]), shape=(n, n))


def main(ref_root):
    os.makedirs(os.path.join(HERE, "_large"), exist_ok=True)
    mats = {}
    for name, dst in (("A_contact", os.path.join(HERE, "A_contact.npz")),
                      ("A_pq", os.path.join(HERE, "_large", "A_pq.npz"))):
        A = scipy.io.mmread(os.path.join(ref_root, "mats", name + ".mtx")).tocsc()
        A.sum_duplicates()
        A.sort_indices()
        np.savez_compressed(dst, indptr=A.indptr.astype(np.int32), indices=A.indices.astype(np.int32),
                            data=A.data.astype(np.float64))
        mats[name] = load_npz(dst)
    out = {}
    meta = {}
    for name, A in mats.items():
        rn_c = O.c_row_l1_norms(A)
        rn_np = O.np_row_l1_norms(A)
        assert np.allclose(rn_c, rn_np, rtol=1e-14, atol=0), name
        out[f"{name}/rn_sum"] = np.array([rn_c.sum()])
        for pname, params in PARAM_SETS.items():
            p = dict(O.DEFAULTS)
            p.update(params)
            sel_c, stats = O.c_gmm_select(rn_c, p["gmm_jump_threshold"], p["gmm_tol"], p["max_gmm_iterations"])
            sel_np, st_np = O.np_gmm_select(rn_np, p["gmm_jump_threshold"], p["gmm_tol"], p["max_gmm_iterations"])
            assert np.array_equal(sel_c, sel_np), (name, pname, len(sel_c), len(sel_np))
            assert stats["gmm_iters"] == st_np["gmm_iters"]
            all_c, subs_c, _ = O.c_select_pipeline(A, params)
            all_np, subs_np = O.np_select_pipeline(A, params)
            assert np.array_equal(all_c, all_np), (name, pname)
            assert len(subs_c) == len(subs_np) and all(np.array_equal(a, b) for a, b in zip(subs_c, subs_np))
            key = f"{name}/{pname}"
            out[key + "/gmm_selection"] = sel_c.astype(np.int32)
            out[key + "/selected"] = all_c.astype(np.int32)
            out[key + "/sub_offsets"] = np.cumsum([0] + [len(s) for s in subs_c]).astype(np.int32)
            meta[key] = {k: (float(v) if isinstance(v, (float, np.floating)) else int(v))
                         for k, v in stats.items()}
            meta[key]["num_subdomains"] = len(subs_c)
            print(key, "gmm", len(sel_c), "selected", len(all_c), "subdomains", len(subs_c),
                  "iters", stats["gmm_iters"], "margin", stats["min_log_margin"])
    np.savez_compressed(os.path.join(HERE, "selection_golden.npz"), **out)
    with open(os.path.join(HERE, "selection_golden.json"), "w") as f:
        json.dump({"param_sets": PARAM_SETS, "stats": meta}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
