"""CPU oracle for the GPU hybrid solve path -- TEST INFRASTRUCTURE ONLY.

Two independent restatements of the reference's stiff-DOF selection
(src/polysolve/linear/GPUHybrid.cu:691-991):

* ``C``   -- ``liblss_oracle.so`` built from ``oracle/lss_oracle.c`` (also holds
  the CPU form of the full method: MAS + stiff-block Cholesky + PCG);
* ``numpy`` -- the functions ``np_*`` below, written separately from the C code.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module; the product never does.

Parity status: the selection is PINNED to the reference's own code.  The
reference ships no golden vectors or known-answer tests for this path and its
solver cannot be built here (hypre, cuDSS, MPI), but its selection stage can:
``oracle/build_ref.py`` compiles GPUHybrid::select_bad_dofs and the three
post-processing passes from the reference sources (thrust host backend) into
``oracle/_ref/libgpuhybrid_ref.so``, wrapped by ``ref_select_pipeline``
below.  tests/golden/ref_selection.npz holds that build's outputs
(tests/golden/make_ref_golden.py), and the CPU tests require the C and numpy
restatements to reproduce them.  The rest of the method (MAS, stiff factor,
PCG) stays a restatement: those parts need hypre / cuDSS / CUDA.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblss_oracle.so")

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class GmmStats(C.Structure):
    _fields_ = [
        ("global_mean", C.c_double), ("global_var", C.c_double),
        ("mean0", C.c_double), ("mean1", C.c_double),
        ("var0", C.c_double), ("var1", C.c_double),
        ("w0", C.c_double), ("w1", C.c_double),
        ("min_log_margin", C.c_double),
        ("gmm_iters", C.c_int32), ("estep_count", C.c_int32),
        ("jump_passed", C.c_int32), ("num_selected", C.c_int32),
    ]


class Params(C.Structure):
    _fields_ = [
        ("max_iter", C.c_int32), ("rel_tol", C.c_double), ("abs_tol", C.c_double),
        ("block_size", C.c_int32), ("do_hybrid", C.c_int32), ("select_from_l1", C.c_int32),
        ("jump_threshold", C.c_double), ("gmm_tol", C.c_double),
        ("max_gmm_iterations", C.c_int32), ("cond_threshold", C.c_double),
        ("decompose", C.c_int32), ("min_sub", C.c_int32), ("max_sub", C.c_int32),
        ("expand", C.c_int32), ("max_coarse_levels", C.c_int32), ("threads", C.c_int32),
        ("additive", C.c_int32), ("mas_omega", C.c_double), ("omega_iters", C.c_int32),
        ("omega_factor", C.c_double), ("greedy_partition", C.c_int32),
    ]


def build(force: bool = False) -> str:
    """Compile liblss_oracle.so in place (gcc, OpenMP)."""
    src = os.path.join(HERE, "lss_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "liblss_oracle.so"],
                       check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.lsso_row_l1_norms.argtypes = [C.c_int32, _i32p, _f64p, _f64p]
        L.lsso_gmm_select.argtypes = [C.c_int32, _f64p, C.c_double, C.c_double, C.c_int32,
                                      _i32p, C.POINTER(GmmStats)]
        L.lsso_gmm_select.restype = C.c_int32
        L.lsso_filter_subdomains.argtypes = [C.c_int32, _i32p, _i32p, _f64p, _i32p, C.c_int32,
                                             C.c_int32, C.c_int32, C.c_double, _i32p, _i32p]
        L.lsso_filter_subdomains.restype = C.c_int32
        L.lsso_expand_subdomains.argtypes = [C.c_int32, _i32p, _i32p, _i32p, C.c_int32, _i32p]
        L.lsso_expand_subdomains.restype = C.c_int32
        L.lsso_decompose_subdomains.argtypes = [C.c_int32, _i32p, _i32p, _i32p, C.c_int32,
                                                C.c_int32, _i32p, _i32p]
        L.lsso_decompose_subdomains.restype = C.c_int32
        L.lsso_mas_create.argtypes = [C.c_int32, C.c_int32, _i32p, _i32p, _f64p, C.c_int32,
                                      _i32p, C.c_int32, _i32p]
        L.lsso_mas_create.restype = C.c_void_p
        L.lsso_mas_apply.argtypes = [C.c_void_p, _f64p, _f64p]
        L.lsso_mas_level_count.argtypes = [C.c_void_p]
        L.lsso_mas_level_count.restype = C.c_int32
        L.lsso_mas_level_items.argtypes = [C.c_void_p, C.c_int32]
        L.lsso_mas_level_items.restype = C.c_int32
        L.lsso_mas_coarse_map.argtypes = [C.c_void_p, C.c_int32, _i32p]
        L.lsso_mas_destroy.argtypes = [C.c_void_p]
        L.lsso_default_params.argtypes = [C.POINTER(Params)]
        L.lsso_params_size.restype = C.c_size_t
        if L.lsso_params_size() != C.sizeof(Params):
            raise RuntimeError("oracle.py Params does not match lsso_params in lss_oracle.h")
        L.lsso_solver_create.argtypes = [C.c_int32, _i32p, _i32p, _f64p, C.POINTER(Params),
                                         _i32p, C.c_int32, _i32p, _i32p]
        L.lsso_solver_create.restype = C.c_void_p
        L.lsso_solver_solve.argtypes = [C.c_void_p, _f64p, _f64p, _i32p, _f64p]
        L.lsso_solver_solve.restype = C.c_int32
        L.lsso_solver_num_stiff.argtypes = [C.c_void_p]
        L.lsso_solver_num_stiff.restype = C.c_int32
        L.lsso_solver_num_subdomains.argtypes = [C.c_void_p]
        L.lsso_solver_num_subdomains.restype = C.c_int32
        L.lsso_solver_precond.argtypes = [C.c_void_p, _f64p, _f64p]
        L.lsso_solver_set_max_iter.argtypes = [C.c_void_p, C.c_int32]
        L.lsso_solver_omega.argtypes = [C.c_void_p]
        L.lsso_solver_omega.restype = C.c_double
        L.lsso_solver_lambda_max.argtypes = [C.c_void_p]
        L.lsso_solver_lambda_max.restype = C.c_double
        L.lsso_tridiag_max_eig.argtypes = [C.c_int32, _f64p, _f64p]
        L.lsso_tridiag_max_eig.restype = C.c_double
        L.lsso_probe_vector.argtypes = [C.c_int32, _f64p]
        L.lsso_solver_destroy.argtypes = [C.c_void_p]
        L.lsso_greedy_partition.argtypes = [C.c_int32, _i32p, _i32p, C.c_int32, _i32p]
        L.lsso_bisect_partition.argtypes = [C.c_int32, _i32p, _i32p, _i32p, _i32p]
        L.lsso_bisect_partition.restype = C.c_int32
        L.lsso_greedy_partition.restype = C.c_int32
        L.lsso_mas_select_elbow.argtypes = [C.c_int32, _f64p, _i32p]
        L.lsso_mas_select_elbow.restype = C.c_int32
        L.lsso_mas_select_kmean.argtypes = [C.c_int32, _f64p, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                            _i32p]
        L.lsso_mas_select_kmean.restype = C.c_int32
        L.lsso_mas_select_gmm.argtypes = [C.c_int32, _f64p, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                          _i32p]
        L.lsso_mas_select_gmm.restype = C.c_int32
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _csc(A):
    """(n, outer, inner, values) int32/float64 contiguous views of a scipy CSC/CSR."""
    outer = np.ascontiguousarray(A.indptr, dtype=np.int32)
    inner = np.ascontiguousarray(A.indices, dtype=np.int32)
    vals = np.ascontiguousarray(A.data, dtype=np.float64)
    return A.shape[0], outer, inner, vals


# --------------------------------------------------------------------------
# C restatement
# --------------------------------------------------------------------------

def c_row_l1_norms(A):
    n, outer, inner, vals = _csc(A)
    out = np.empty(n, np.float64)
    lib().lsso_row_l1_norms(n, _p(outer, _i32p), _p(vals, _f64p), _p(out, _f64p))
    return out


def c_gmm_select(rn, jump_threshold=100.0, tol=1e-3, max_iterations=20):
    rn = np.ascontiguousarray(rn, dtype=np.float64)
    sel = np.empty(max(len(rn), 1), np.int32)
    st = GmmStats()
    k = lib().lsso_gmm_select(len(rn), _p(rn, _f64p), jump_threshold, tol, max_iterations,
                              _p(sel, _i32p), C.byref(st))
    stats = {f: getattr(st, f) for f, _ in GmmStats._fields_}
    return sel[:k].copy(), stats


def c_mas_select(strategy, score, p1=0.0, p2=0.0, i1=0, i2=0):
    """MASSolver's bad-DOF selections (lss_oracle.c): "elbow" on |diagonal|
    (BadDOFPreconditioner.cu:61-100), "kmean" (p1 search fraction, p2 jump
    threshold, i1 iterations, i2 expand neighbours; BadDofKMeanPreconditioner.cu:63-172),
    "gmm" (p1 jump threshold, p2 tol, i1 iterations, i2 expand neighbours;
    BadDofGMMPreconditioner.cu:73-255).  Positions in the reference's output order."""
    v = np.ascontiguousarray(score, np.float64)
    out = np.empty(max(len(v), 1), np.int32)
    L = lib()
    if strategy == "elbow":
        k = L.lsso_mas_select_elbow(len(v), _p(v, _f64p), _p(out, _i32p))
    elif strategy == "kmean":
        k = L.lsso_mas_select_kmean(len(v), _p(v, _f64p), p1, p2, i1, i2, _p(out, _i32p))
    else:
        k = L.lsso_mas_select_gmm(len(v), _p(v, _f64p), p1, p2, i1, i2, _p(out, _i32p))
    return out[:k].copy()


def c_filter(A, sel, min_size=1, max_size=10000000, cond=100.0):
    n, outer, inner, vals = _csc(A)
    sel = np.ascontiguousarray(sel, dtype=np.int32)
    out = np.empty(max(len(sel), 1), np.int32)
    cnt = np.zeros(3, np.int32)
    k = lib().lsso_filter_subdomains(n, _p(outer, _i32p), _p(inner, _i32p), _p(vals, _f64p),
                                     _p(sel, _i32p), len(sel), min_size, max_size, cond,
                                     _p(out, _i32p), _p(cnt, _i32p))
    return out[:k].copy(), cnt


def c_expand(A, sel):
    n, outer, inner, _ = _csc(A)
    sel = np.ascontiguousarray(sel, dtype=np.int32)
    out = np.empty(max(n, 1), np.int32)
    k = lib().lsso_expand_subdomains(n, _p(outer, _i32p), _p(inner, _i32p), _p(sel, _i32p),
                                     len(sel), _p(out, _i32p))
    return out[:k].copy()


def c_decompose(A, sel, max_size=10000000):
    n, outer, inner, _ = _csc(A)
    sel = np.ascontiguousarray(sel, dtype=np.int32)
    offs = np.empty(len(sel) + 1, np.int32)
    dofs = np.empty(max(len(sel), 1), np.int32)
    k = lib().lsso_decompose_subdomains(n, _p(outer, _i32p), _p(inner, _i32p), _p(sel, _i32p),
                                        len(sel), max_size, _p(offs, _i32p), _p(dofs, _i32p))
    return [dofs[offs[i]:offs[i + 1]].copy() for i in range(k)]


def c_select_pipeline(A, params: dict):
    """GPUHybrid::factorize selection stage (GPUHybrid.cu:214-238)."""
    p = dict(DEFAULTS)
    p.update(params)
    if not p["do_hybrid_precond"]:
        return np.zeros(0, np.int32), [], {}
    stats = {}
    sel = np.zeros(0, np.int32)
    if p["select_bad_dofs_from_l1_norm"]:
        rn = c_row_l1_norms(A)
        sel, stats = c_gmm_select(rn, p["gmm_jump_threshold"], p["gmm_tol"], p["max_gmm_iterations"])
    stats["num_selected_gmm"] = len(sel)
    if p["decompose_subdomains"]:
        sel, cnt = c_filter(A, sel, p["min_subdomain_size"], p["max_subdomain_size"],
                            p["conditioning_threshold"])
        stats["filter_counters"] = cnt.tolist()
    if p["expand_subdomains"] and len(sel):
        sel = c_expand(A, sel)
    if p["decompose_subdomains"]:
        subs = c_decompose(A, sel, p["max_subdomain_size"])
    else:
        subs = [sel.copy()] if len(sel) else []
    allsel = np.sort(np.concatenate(subs)) if subs else np.zeros(0, np.int32)
    return allsel.astype(np.int32), subs, stats


# --------------------------------------------------------------------------
# numpy restatement (independent of the C code)
# --------------------------------------------------------------------------

DEFAULTS = {
    # linear-solver-spec.json:646-747 (/GPUHybrid defaults)
    "max_iter": 10000, "relative_tolerance": 1e-10, "absolute_tolerance": 0.0,
    "block_size": 1, "theta": 0.5, "do_hybrid_precond": True,
    "select_bad_dofs_from_l1_norm": True, "conditioning_threshold": 100.0,
    "gmm_jump_threshold": 100.0, "gmm_tol": 1e-3, "max_gmm_iterations": 20,
    "decompose_subdomains": True, "min_subdomain_size": 1, "max_subdomain_size": 10000000,
    "expand_subdomains": True, "max_dense_size": 0, "use_float_on_subdomains": False,
}


def np_row_l1_norms(A):
    """GPUHybrid.cu:753-765: sum of |a| over each outer slice."""
    out = np.zeros(A.shape[0])
    lens = np.diff(A.indptr)
    nz = lens > 0
    out[nz] = np.add.reduceat(np.abs(A.data), A.indptr[:-1][nz])
    return out


def np_gmm_select(rn, jump_threshold=100.0, tol=1e-3, max_iterations=20):
    """GPUHybrid.cu:767-879 (EM for a two-component 1D GMM, log-space E-step)."""
    rn = np.asarray(rn, np.float64)
    n = len(rn)
    mean = rn.sum() / n
    var = ((rn - mean) ** 2).sum() / n
    m0, m1, v0, v1, w0, w1 = rn.min(), rn.max(), var, var, 0.5, 0.5
    g0 = np.zeros(n)
    g1 = np.zeros(n)
    it = 0
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        while it < max_iterations:
            lg0 = math.log(w0) + (-0.5 * np.log(2.0 * np.pi * v0) - 0.5 * (rn - m0) * (rn - m0) / v0)
            lg1 = math.log(w1) + (-0.5 * np.log(2.0 * np.pi * v1) - 0.5 * (rn - m1) * (rn - m1) / v1)
            mx = np.fmax(lg0, lg1)
            lt = mx + np.log(np.exp(lg0 - mx) + np.exp(lg1 - mx))
            g0 = np.exp(lg0 - lt)
            g1 = np.exp(lg1 - lt)
            s0, s1 = g0.sum(), g1.sum()
            w0, w1 = s0 / n, s1 / n
            om0, om1, ov0, ov1 = m0, m1, v0, v1
            m0 = (g0 * rn).sum() / s0
            m1 = (g1 * rn).sum() / s1
            v0 = (g0 * (rn - m0) * (rn - m0)).sum() / s0 + 1e-6
            v1 = (g1 * (rn - m1) * (rn - m1)).sum() / s1 + 1e-6
            if (abs(m0 - om0) / abs(om0) < tol and abs(m1 - om1) / abs(om1) < tol
                    and abs(v0 - ov0) / abs(ov0) < tol and abs(v1 - ov1) / abs(ov1) < tol):
                break
            it += 1
        jump = abs(m1) / abs(m0) > jump_threshold
    sel = np.nonzero(g0 < g1)[0].astype(np.int32) if jump else np.zeros(0, np.int32)
    return sel, {"mean0": m0, "mean1": m1, "var0": v0, "var1": v1, "gmm_iters": it,
                 "jump_passed": bool(jump)}


def _np_components(A, sel):
    """Connected components of sel in A's pattern (outer slice k holds row ids)."""
    import scipy.sparse as sp
    import scipy.sparse.csgraph as csg
    sel = np.asarray(sel, np.int64)
    if len(sel) == 0:
        return []
    sub = A[sel][:, sel] if sp.isspmatrix_csr(A) else A.tocsr()[sel][:, sel]
    nc, lab = csg.connected_components(sub, directed=True, connection="weak")
    comps = [sel[lab == c] for c in range(nc)]
    comps.sort(key=lambda c: c[0])
    return comps


def np_filter(A, sel, min_size=1, max_size=10000000, cond=100.0):
    """GPUHybrid.cu:885-970."""
    sel = np.asarray(sel, np.int64)
    inset = np.zeros(A.shape[0], bool)
    inset[sel] = True
    Ac = A.tocsc()
    keep = []
    for comp in _np_components(A, sel):
        if len(comp) < min_size or len(comp) > max_size:
            continue
        lmin, lmax = np.finfo(np.float64).max, 0.0
        for k in comp:
            rows = Ac.indices[Ac.indptr[k]:Ac.indptr[k + 1]]
            vals = Ac.data[Ac.indptr[k]:Ac.indptr[k + 1]]
            m = inset[rows]
            d = vals[m & (rows == k)]
            diag = d[-1] if len(d) else 0.0
            off = np.abs(vals[m & (rows != k)]).sum()
            lmin = min(lmin, diag - off)
            lmax = max(lmax, diag + off)
        with np.errstate(divide="ignore", invalid="ignore"):
            if lmin * lmax < 0.0 or lmax / lmin > cond:
                keep.append(comp)
    return np.sort(np.concatenate(keep)).astype(np.int32) if keep else np.zeros(0, np.int32)


def np_expand(A, sel):
    """GPUHybrid.cu:972-991."""
    Ac = A.tocsc()
    sel = np.asarray(sel, np.int64)
    if len(sel) == 0:
        return np.zeros(0, np.int32)
    rows = np.concatenate([Ac.indices[Ac.indptr[k]:Ac.indptr[k + 1]] for k in sel])
    return np.unique(rows).astype(np.int32)


def np_select_pipeline(A, params: dict):
    p = dict(DEFAULTS)
    p.update(params)
    if not p["do_hybrid_precond"]:
        return np.zeros(0, np.int32), []
    A = A.tocsc()
    A.sort_indices()
    sel = np.zeros(0, np.int32)
    if p["select_bad_dofs_from_l1_norm"]:
        sel, _ = np_gmm_select(np_row_l1_norms(A), p["gmm_jump_threshold"], p["gmm_tol"],
                               p["max_gmm_iterations"])
    if p["decompose_subdomains"]:
        sel = np_filter(A, sel, p["min_subdomain_size"], p["max_subdomain_size"],
                        p["conditioning_threshold"])
    if p["expand_subdomains"] and len(sel):
        sel = np_expand(A, sel)
    if p["decompose_subdomains"]:
        subs = [c.astype(np.int32) for c in _np_components(A, sel)
                if len(c) <= p["max_subdomain_size"]]
    else:
        subs = [np.asarray(sel, np.int32)] if len(sel) else []
    allsel = np.sort(np.concatenate(subs)).astype(np.int32) if subs else np.zeros(0, np.int32)
    return allsel, subs


# --------------------------------------------------------------------------
# MAS and the full CPU method
# --------------------------------------------------------------------------

class Mas:
    """lsso_mas: MASPreconditioner on a partition-ordered block CSR."""

    def __init__(self, nb, bd, rows, cols, vals, part_offsets, max_coarse_levels=4):
        self._keep = [np.ascontiguousarray(rows, np.int32), np.ascontiguousarray(cols, np.int32),
                      np.ascontiguousarray(vals, np.float64),
                      np.ascontiguousarray(part_offsets, np.int32)]
        r, c, v, po = self._keep
        st = C.c_int32(0)
        self.h = lib().lsso_mas_create(nb, bd, _p(r, _i32p), _p(c, _i32p), _p(v, _f64p),
                                       len(po) - 1, _p(po, _i32p), max_coarse_levels, C.byref(st))
        self.status = st.value
        self.nb, self.bd = nb, bd

    def levels(self):
        return lib().lsso_mas_level_count(self.h)

    def level_items(self, l):
        return lib().lsso_mas_level_items(self.h, l)

    def coarse_map(self, l):
        out = np.empty(self.nb, np.int32)
        lib().lsso_mas_coarse_map(self.h, l, _p(out, _i32p))
        return out

    def apply(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.empty_like(r)
        lib().lsso_mas_apply(self.h, _p(r, _f64p), _p(z, _f64p))
        return z

    def __del__(self):
        if getattr(self, "h", None):
            lib().lsso_mas_destroy(self.h)
            self.h = None


def make_params(params: dict, threads=0, max_coarse_levels=4, additive=False, mas_omega=0.0,
                omega_iters=20, omega_factor=1.5, greedy_partition=False) -> Params:
    p = dict(DEFAULTS)
    p.update(params)
    P = Params()
    lib().lsso_default_params(C.byref(P))
    P.max_iter = int(p["max_iter"])
    P.rel_tol = float(p["relative_tolerance"])
    P.abs_tol = float(p["absolute_tolerance"])
    P.block_size = int(p["block_size"])
    P.do_hybrid = int(bool(p["do_hybrid_precond"]))
    P.select_from_l1 = int(bool(p["select_bad_dofs_from_l1_norm"]))
    P.jump_threshold = float(p["gmm_jump_threshold"])
    P.gmm_tol = float(p["gmm_tol"])
    P.max_gmm_iterations = int(p["max_gmm_iterations"])
    P.cond_threshold = float(p["conditioning_threshold"])
    P.decompose = int(bool(p["decompose_subdomains"]))
    P.min_sub = int(p["min_subdomain_size"])
    P.max_sub = int(p["max_subdomain_size"])
    P.expand = int(bool(p["expand_subdomains"]))
    P.max_coarse_levels = int(max_coarse_levels)
    P.threads = int(threads)
    P.additive = int(bool(additive))
    P.mas_omega = float(mas_omega)
    P.omega_iters = int(omega_iters)
    P.omega_factor = float(omega_factor)
    P.greedy_partition = int(bool(greedy_partition))
    return P


class CpuSolver:
    """The full method on the CPU (selection, MAS, stiff Cholesky, PCG)."""

    def __init__(self, A, params: dict, perm=None, part_offsets=None, threads=0,
                 max_coarse_levels=4, additive=False, mas_omega=0.0, omega_iters=20, omega_factor=1.5):
        n, outer, inner, vals = _csc(A)
        self._keep = [outer, inner, vals]
        P = make_params(params, threads, max_coarse_levels, additive, mas_omega, omega_iters,
                        omega_factor)
        st = C.c_int32(0)
        if perm is not None:
            perm = np.ascontiguousarray(perm, np.int32)
            part_offsets = np.ascontiguousarray(part_offsets, np.int32)
            self._keep += [perm, part_offsets]
            pp, npart, po = _p(perm, _i32p), len(part_offsets) - 1, _p(part_offsets, _i32p)
        else:
            pp, npart, po = None, 0, None
        self.h = lib().lsso_solver_create(n, _p(outer, _i32p), _p(inner, _i32p), _p(vals, _f64p),
                                          C.byref(P), pp, npart, po, C.byref(st))
        self.status = st.value
        self.n = n

    @property
    def num_stiff(self):
        return lib().lsso_solver_num_stiff(self.h)

    @property
    def omega(self):
        return lib().lsso_solver_omega(self.h)

    @property
    def lambda_max(self):
        return lib().lsso_solver_lambda_max(self.h)

    @property
    def num_subdomains(self):
        return lib().lsso_solver_num_subdomains(self.h)

    def precond(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.empty_like(r)
        lib().lsso_solver_precond(self.h, _p(r, _f64p), _p(z, _f64p))
        return z

    def solve(self, b, x0=None):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.n) if x0 is None else np.array(x0, np.float64, copy=True)
        it = C.c_int32(0)
        res = C.c_double(0)
        code = lib().lsso_solver_solve(self.h, _p(b, _f64p), _p(x, _f64p), C.byref(it), C.byref(res))
        return x, {"num_iterations": it.value, "final_res_norm": res.value, "code": code}

    def __del__(self):
        if getattr(self, "h", None):
            lib().lsso_solver_destroy(self.h)
            self.h = None


# --------------------------------------------------------------------------
# the reference's own selection code, compiled on the host (oracle/build_ref.py)
# --------------------------------------------------------------------------

_ref_lib = None


def greedy_partition(G, max_part=32):
    """The oracle's greedy breadth-first partition (lsso_greedy_partition) of
    a block graph G (scipy CSR, no self loops): (perm[old] = new, offsets)."""
    G = G.tocsr()
    nb = G.shape[0]
    rows = np.ascontiguousarray(G.indptr, np.int32)
    cols = np.ascontiguousarray(G.indices, np.int32)
    part_of = np.zeros(max(nb, 1), np.int32)
    nparts = lib().lsso_greedy_partition(nb, _p(rows, _i32p), _p(cols, _i32p), max_part, _p(part_of, _i32p))
    part_of = part_of[:nb]
    counts = np.bincount(part_of, minlength=nparts)
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    order = np.argsort(part_of, kind="stable")
    perm = np.empty(nb, np.int32)
    perm[order] = np.arange(nb, dtype=np.int32)
    return perm, offs


def bisect_partition(G):
    """The library's partition restated in C (lsso_bisect_partition) on a
    block graph G (scipy CSR): (perm[old] = new, part_offsets)."""
    G = G.tocsr()
    nb = G.shape[0]
    rows = np.ascontiguousarray(G.indptr, np.int32)
    cols = np.ascontiguousarray(G.indices, np.int32)
    perm = np.zeros(max(nb, 1), np.int32)
    offs = np.zeros(nb + 2, np.int32)
    np_ = lib().lsso_bisect_partition(nb, _p(rows, _i32p), _p(cols, _i32p), _p(perm, _i32p), _p(offs, _i32p))
    return perm[:nb].copy(), offs[:np_ + 1].copy()


def ref_lib():
    """oracle/_ref/libgpuhybrid_ref.so, built on first use; None when neither
    the reference checkout nor its extracted sources are present."""
    global _ref_lib
    if _ref_lib is None:
        from oracle import build_ref
        path = build_ref.build()
        if path is None:
            return None
        L = C.CDLL(path)
        L.lssref_select.argtypes = [C.c_int32, _i32p, _i32p, _f64p, C.c_double, C.c_double, C.c_int32,
                                    C.c_double, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    _i32p, _i32p, _i32p, _i32p, _i32p, _f64p, C.c_char_p, C.c_int32]
        L.lssref_select.restype = C.c_int32
        _ref_lib = L
    return _ref_lib


def ref_select_pipeline(A, params: dict):
    """GPUHybrid::factorize's selection stage run by the reference's own code
    (GPUHybrid.cu:215-238 orchestrating :691-991).  Returns the GMM selection,
    the subdomains in the reference's order, and the GMM statistics of its
    "[bad_dof_selection]" log line."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("the reference build (oracle/_ref) is not available")
    p = dict(DEFAULTS)
    p.update(params)
    n, indptr, indices, data = _csc(A)
    raw = np.zeros(max(n, 1), np.int32)
    sub_off = np.zeros(n + 2, np.int32)
    sub_dofs = np.zeros(max(n, 1), np.int32)
    nraw, nsub = C.c_int32(0), C.c_int32(0)
    stats = np.zeros(8)
    err = C.create_string_buffer(512)
    st = L.lssref_select(n, _p(indptr, _i32p), _p(indices, _i32p), _p(data, _f64p), p["gmm_jump_threshold"],
                         p["gmm_tol"], p["max_gmm_iterations"], p["conditioning_threshold"],
                         int(p["decompose_subdomains"]), p["min_subdomain_size"], p["max_subdomain_size"],
                         int(p["expand_subdomains"]), _p(raw, _i32p), C.byref(nraw), _p(sub_off, _i32p),
                         _p(sub_dofs, _i32p), C.byref(nsub), _p(stats, _f64p), err, 512)
    if st != 0:
        raise RuntimeError("reference selection failed: " + err.value.decode())
    subs = [sub_dofs[sub_off[k]:sub_off[k + 1]].copy() for k in range(nsub.value)]
    keys = ["global_mean", "global_var", "mean0", "mean1", "var0", "var1", "gmm_iters", "num_selected"]
    return raw[:nraw.value].copy(), subs, dict(zip(keys, stats.tolist()))
