"""Python mirror of the reference's linear-solver interface over the C ABI.

``Solver.create(params)`` / ``set_parameters`` / ``get_info`` /
``analyze_pattern`` / ``factorize`` / ``solve`` / ``name`` /
``set_problematic_dofs`` keep the names, argument meaning and error
behaviour of ``polysolve::linear::Solver`` (src/polysolve/linear/Solver.hpp:
32-149) for the ``GPUHybrid`` solver (GPUHybrid.hpp:27-192).  Matrices are
scipy sparse matrices (CSC as in Eigen's ``StiffnessMatrix``; a CSR matrix is
accepted too, its outer index taken as the row like the reference does), vectors
numpy float64 arrays.  Every call goes through ``liblss.so``; a missing
library raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _paths

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)

STATUS = {
    0: "LSS_OK", 1: "LSS_ERR_INVALID_ARGUMENT", 2: "LSS_ERR_CUDA", 3: "LSS_ERR_OOM",
    4: "LSS_ERR_NOT_FACTORIZED", 5: "LSS_ERR_NOT_SPD", 6: "LSS_ERR_NONFINITE", 7: "LSS_ERR_INTERNAL",
    8: "LSS_ERR_BUFFER_TOO_SMALL", 9: "LSS_ERR_NO_DEVICE", 10: "LSS_ERR_UNSUPPORTED",
}

# symbols declared in include/lss.h
EXPORTS = [
    "lss_status_string", "lss_last_error", "lss_create", "lss_destroy", "lss_set_parameters",
    "lss_get_info", "lss_name", "lss_analyze_pattern", "lss_factorize", "lss_factorize_device",
    "lss_set_problematic_dofs",
    "lss_solve", "lss_solve_device", "lss_solve_transpose", "lss_grad_A_pattern",
    "lss_grad_A_pattern_device", "lss_grad_params_device", "lss_selected_dofs", "lss_gmm_selection", "lss_subdomains",
    "lss_partition", "lss_op_row_l1_norms", "lss_op_spmv", "lss_op_spmv_outer", "lss_op_mas_apply", "lss_op_precond",
    "lss_op_time", "lss_set_memory_cap", "lss_gmm_select_device_noalloc", "lss_solve_batched_device",
    "lss_factorize_batched_device", "lss_op_row_scores", "lss_op_select_bad_dofs", "lss_partition_pattern",
    "lss_batch_create", "lss_batch_destroy", "lss_batch_last_error", "lss_batch_factorize_device",
    "lss_batch_solve_device", "lss_batch_get_info", "lss_assemble_values_device", "lss_stiff_elimination_tree",
    "lss_postprocess_selection", "lss_coarse_space", "lss_stiff_elimination_plan",
]

BATCH_RHS = 16


class LssError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code
        self.status = STATUS.get(code, str(code))


_lib = None


def load(path: str | None = None):
    """Load liblss.so (built in-tree by lss.build.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or _paths.lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: the CUDA library must be built (lss.build.build())")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.lss_status_string.restype = C.c_char_p
    L.lss_status_string.argtypes = [C.c_int]
    L.lss_last_error.restype = C.c_char_p
    L.lss_last_error.argtypes = [vp]
    L.lss_create.argtypes = [C.c_char_p, C.POINTER(vp)]
    L.lss_destroy.argtypes = [vp]
    L.lss_set_parameters.argtypes = [vp, C.c_char_p]
    L.lss_get_info.argtypes = [vp, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]
    L.lss_name.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.lss_partition_pattern.argtypes = [C.c_int32, C.c_int64, _i32p, _i32p, C.c_int32, C.c_int32, _i32p, C.c_int32,
                                        _i32p, C.c_int32, _i32p]
    L.lss_analyze_pattern.argtypes = [vp, C.c_int32, C.c_int64, _i32p, _i32p]
    L.lss_factorize.argtypes = [vp, C.c_int32, C.c_int64, _i32p, _i32p, _f64p]
    L.lss_factorize_device.argtypes = [vp, vp, vp]
    L.lss_set_problematic_dofs.argtypes = [vp, _i32p, C.c_int32]
    L.lss_solve.argtypes = [vp, _f64p, _f64p, C.c_int32, C.c_int64]
    L.lss_solve_device.argtypes = [vp, vp, vp, vp]
    L.lss_solve_transpose.argtypes = [vp, _f64p, _f64p]
    L.lss_grad_A_pattern.argtypes = [vp, _f64p, _f64p, _f64p]
    L.lss_grad_A_pattern_device.argtypes = [vp, vp, vp, vp, vp]
    L.lss_grad_params_device.argtypes = [vp, vp, vp, C.c_int32, vp, vp, vp, vp, vp]
    L.lss_selected_dofs.argtypes = [vp, _i32p, C.c_int32, _i32p]
    L.lss_gmm_selection.argtypes = [vp, _i32p, C.c_int32, _i32p]
    L.lss_subdomains.argtypes = [vp, _i32p, C.c_int32, _i32p, C.c_int32, _i32p, _i32p]
    L.lss_partition.argtypes = [vp, _i32p, C.c_int32, _i32p, C.c_int32, _i32p]
    L.lss_op_row_l1_norms.argtypes = [C.c_int32, C.c_int64, _i32p, _f64p, _f64p]
    L.lss_op_spmv.argtypes = [vp, _f64p, _f64p]
    L.lss_op_spmv_outer.argtypes = [vp, _f64p, _f64p]
    L.lss_op_mas_apply.argtypes = [vp, _f64p, _f64p]
    L.lss_op_precond.argtypes = [vp, _f64p, _f64p]
    L.lss_op_time.argtypes = [vp, C.c_int32, C.c_int32, _f64p, _f64p]
    L.lss_set_memory_cap.argtypes = [C.c_size_t]
    L.lss_solve_batched_device.argtypes = [C.POINTER(vp), C.c_int32, C.POINTER(vp), C.POINTER(vp), C.c_int32,
                                           C.c_int32, _i32p]
    L.lss_factorize_batched_device.argtypes = [C.POINTER(vp), C.c_int32, C.POINTER(vp), C.c_int32]
    L.lss_op_row_scores.argtypes = [vp, _f64p, _f64p, _f64p]
    L.lss_op_select_bad_dofs.argtypes = [C.c_int32, C.c_int32, _f64p, C.c_double, C.c_double, C.c_int32,
                                         C.c_int32, _i32p, _i32p]
    L.lss_gmm_select_device_noalloc.argtypes = [C.c_int32, C.c_int64, vp, vp, C.c_double, C.c_double, C.c_int32,
                                                vp, vp, vp]
    L.lss_assemble_values_device.argtypes = [C.c_int64, vp, vp, vp, vp, vp, vp, vp]
    L.lss_batch_create.argtypes = [C.POINTER(vp), C.c_int32, C.POINTER(vp)]
    L.lss_batch_destroy.argtypes = [vp]
    L.lss_batch_last_error.argtypes = [vp]
    L.lss_batch_last_error.restype = C.c_char_p
    L.lss_batch_factorize_device.argtypes = [vp, C.POINTER(vp), C.c_int32]
    L.lss_batch_solve_device.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), _i32p]
    L.lss_batch_get_info.argtypes = [vp, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]
    for name in EXPORTS:
        fn = getattr(L, name)
        if fn.restype is C.c_int or fn.restype is None:
            if name not in ("lss_status_string", "lss_last_error", "lss_batch_last_error"):
                fn.restype = C.c_int
    if path == _paths.lib_path():
        _lib = L
    return L


def _p(a, t):
    return a.ctypes.data_as(t)


def _csc_arrays(A):
    import scipy.sparse as sp
    if not sp.issparse(A):
        raise TypeError("A must be a scipy sparse matrix")
    if A.format not in ("csc", "csr"):
        A = A.tocsc()
    if not A.has_canonical_format:
        A = A.copy()
        A.sum_duplicates()
    outer = np.ascontiguousarray(A.indptr, np.int32)
    inner = np.ascontiguousarray(A.indices, np.int32)
    vals = np.ascontiguousarray(A.data, np.float64)
    return A.shape[0], outer, inner, vals


def row_l1_norms(A):
    """GPU l1 row norms of A's outer slices (GPUHybrid.cu:753-765)."""
    L = load()
    n, outer, _, vals = _csc_arrays(A)
    out = np.empty(n)
    st = L.lss_op_row_l1_norms(n, len(vals), _p(outer, _i32p), _p(vals, _f64p), _p(out, _f64p))
    if st:
        raise LssError(st, L.lss_last_error(None).decode())
    return out


def partition_pattern(A, block_size: int, threads: int = 0):
    """The MAS partition of A's block graph, computed on the host
    (lss_partition_pattern): (perm[old block] = new block, part_offsets)."""
    L = load()
    n, outer, inner, _ = _csc_arrays(A)
    nparts = C.c_int32(0)
    nb = n // block_size
    perm = np.zeros(max(nb, 1), np.int32)
    offs = np.zeros(nb + 2, np.int32)
    st = L.lss_partition_pattern(n, len(inner), _p(outer, _i32p), _p(inner, _i32p), block_size, threads,
                                 _p(perm, _i32p), len(perm), _p(offs, _i32p), len(offs), C.byref(nparts))
    if st != 0:
        raise LssError(st, L.lss_last_error(None).decode())
    return perm[:nb].copy(), offs[:nparts.value + 1].copy()


def postprocess_selection(A, params: dict, sel):
    """The solver's post-processing of a stiff-DOF selection, on the host
    (lss_postprocess_selection): filter, one-ring expansion, decomposition.
    params: the "GPUHybrid" parameters.  Returns the subdomains (ascending
    arrays, ordered by first DOF)."""
    import json as _json
    L = load()
    n, outer, inner, vals = _csc_arrays(A)
    s = np.ascontiguousarray(np.asarray(sel, np.int32))
    cfg = _json.dumps({"solver": "GPUHybrid", "GPUHybrid": dict(params)}).encode()
    nsub = C.c_int32(0)
    off = np.zeros(n + 1, np.int32)
    dofs = np.zeros(max(n, 1), np.int32)
    st = L.lss_postprocess_selection(n, len(inner), _p(outer, _i32p), _p(inner, _i32p),
                                     vals.ctypes.data_as(C.POINTER(C.c_double)), cfg, _p(s, _i32p), len(s),
                                     _p(off, _i32p), len(off), _p(dofs, _i32p), len(dofs), C.byref(nsub))
    if st != 0:
        raise LssError(st, L.lss_last_error(None).decode())
    k = nsub.value
    return [dofs[off[q]:off[q + 1]].copy() for q in range(k)]


def coarse_space(A, block_size: int, max_coarse_levels: int = 4):
    """The MAS coarse space of A's pattern (lss_coarse_space, host only):
    (items per level, [cmap of level l for l = 1 .. L-1] over the permuted
    block rows)."""
    L = load()
    n, outer, inner, _ = _csc_arrays(A)
    nb = n // block_size
    lev = C.c_int32(0)
    items = np.zeros(16, np.int32)
    cmap = np.zeros(max(16 * nb, 1), np.int32)
    st = L.lss_coarse_space(n, len(inner), _p(outer, _i32p), _p(inner, _i32p), block_size, max_coarse_levels,
                            C.byref(lev), _p(items, _i32p), len(items), _p(cmap, _i32p), C.c_int64(len(cmap)))
    if st != 0:
        raise LssError(st, L.lss_last_error(None).decode())
    k = lev.value
    return items[:k].copy(), [cmap[(l - 1) * nb:l * nb].copy() for l in range(1, k)]


def stiff_elimination_plan(A, block_size: int, dofs) -> dict:
    """The full multifrontal plan for one stiff subdomain
    (lss_stiff_elimination_plan, host only): per front (postorder) its first
    position, own and boundary counts, boundary positions and children, and
    pos2j (position -> index into dofs)."""
    L = load()
    n, outer, inner, _ = _csc_arrays(A)
    d = np.ascontiguousarray(np.sort(np.asarray(dofs, np.int32)))
    counts = np.zeros(4, np.int64)
    args = [n, len(inner), _p(outer, _i32p), _p(inner, _i32p), block_size, _p(d, _i32p), len(d),
            counts.ctypes.data_as(C.POINTER(C.c_int64))]
    st = L.lss_stiff_elimination_plan(*args, *([None] * 8))
    if st != 0:
        raise LssError(st, L.lss_last_error(None).decode())
    nf, npos, nb_, nc = (int(v) for v in counts)
    arr = {"p0": np.zeros(nf, np.int32), "s": np.zeros(nf, np.int32), "u": np.zeros(nf, np.int32),
           "bnd_off": np.zeros(nf + 1, np.int32), "bnd_pos": np.zeros(max(nb_, 1), np.int32),
           "child_off": np.zeros(nf + 1, np.int32), "child": np.zeros(max(nc, 1), np.int32),
           "pos2j": np.zeros(npos, np.int32)}
    st = L.lss_stiff_elimination_plan(*args, *[_p(arr[k], _i32p) for k in
                                               ("p0", "s", "u", "bnd_off", "bnd_pos", "child_off", "child", "pos2j")])
    if st != 0:
        raise LssError(st, L.lss_last_error(None).decode())
    arr["bnd_pos"] = arr["bnd_pos"][:nb_]
    arr["child"] = arr["child"][:nc]
    return arr


def stiff_elimination_tree(A, block_size: int, dofs) -> dict:
    """The multifrontal plan for one stiff subdomain (lss_stiff_elimination_tree,
    host only): fronts, tree levels, largest front, factorization FMAs."""
    L = load()
    n, outer, inner, _ = _csc_arrays(A)
    d = np.ascontiguousarray(np.sort(np.asarray(dofs, np.int32)))
    out = np.zeros(4, np.float64)
    st = L.lss_stiff_elimination_tree(n, len(inner), _p(outer, _i32p), _p(inner, _i32p), block_size,
                                      _p(d, _i32p), len(d), out.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise LssError(st, L.lss_last_error(None).decode())
    return {"fronts": int(out[0]), "levels": int(out[1]), "max_front": int(out[2]), "fmas": float(out[3])}


def solve_batched_device(solvers, d_b, d_x, nrhs: int, threads: int = 0) -> np.ndarray:
    """Solve every system s (a factorized Solver) for nrhs right-hand sides at
    once: d_b[s], d_x[s] are device pointers (ints) to n_s x nrhs column-major
    arrays; x is the initial guess on entry.  One host thread per system
    (threads <= 0) drives that solver's PCG on its own stream, so the GPU
    overlaps the systems.  Returns the iteration counts, shape (count, nrhs)."""
    L = load()
    count = len(solvers)
    if len(d_b) != count or len(d_x) != count:
        raise ValueError("one b and one x pointer per system")
    S = (C.c_void_p * max(count, 1))(*[s._h.value for s in solvers])
    B = (C.c_void_p * max(count, 1))(*[int(p) for p in d_b])
    X = (C.c_void_p * max(count, 1))(*[int(p) for p in d_x])
    its = np.zeros(max(count * nrhs, 1), np.int32)
    st = L.lss_solve_batched_device(S, count, B, X, nrhs, threads, _p(its, _i32p))
    if st:
        raise LssError(st, L.lss_last_error(None).decode())
    return its[:count * nrhs].reshape(count, nrhs)


def factorize_batched_device(solvers, d_values, threads: int = 0) -> None:
    """factorize_device of every system at once (d_values[s]: device pointer to
    system s's values in its analysed pattern's CSC order)."""
    L = load()
    count = len(solvers)
    if len(d_values) != count:
        raise ValueError("one values pointer per system")
    S = (C.c_void_p * max(count, 1))(*[s._h.value for s in solvers])
    V = (C.c_void_p * max(count, 1))(*[int(p) for p in d_values])
    st = L.lss_factorize_batched_device(S, count, V, threads)
    if st:
        raise LssError(st, L.lss_last_error(None).decode())


class Batch:
    """Batched PCG over factorized solvers (lss_batch_*): every step is one
    launch per kernel over all systems and BATCH_RHS right-hand sides each."""

    def __init__(self, solvers):
        self._L = load()
        self._h = C.c_void_p()
        self._solvers = list(solvers)  # the batch reads their factorizations
        S = (C.c_void_p * len(self._solvers))(*[s._h.value for s in self._solvers])
        st = self._L.lss_batch_create(S, len(self._solvers), C.byref(self._h))
        if st:
            raise LssError(st, self._L.lss_batch_last_error(None).decode())

    def _check(self, st):
        if st:
            raise LssError(st, self._L.lss_batch_last_error(self._h).decode())

    def factorize_device(self, d_values, threads: int = 0):
        V = (C.c_void_p * len(self._solvers))(*[int(p) for p in d_values])
        self._check(self._L.lss_batch_factorize_device(self._h, V, threads))

    def solve_device(self, d_b, d_x) -> np.ndarray:
        """d_b[s], d_x[s]: device pointers to n_s x BATCH_RHS column-major
        arrays (x: initial guess in, solution out).  Returns the iterations,
        shape (count, BATCH_RHS)."""
        n = len(self._solvers)
        B = (C.c_void_p * n)(*[int(p) for p in d_b])
        X = (C.c_void_p * n)(*[int(p) for p in d_x])
        its = np.zeros(n * BATCH_RHS, np.int32)
        self._check(self._L.lss_batch_solve_device(self._h, B, X, _p(its, _i32p)))
        return its.reshape(n, BATCH_RHS)

    def get_info(self) -> dict:
        n = C.c_size_t(0)
        self._L.lss_batch_get_info(self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value + 1)
        self._check(self._L.lss_batch_get_info(self._h, buf, n.value + 1, C.byref(n)))
        return json.loads(buf.value.decode())

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.lss_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


BAD_DOF_STRATEGIES = {"elbow": 1, "kmean": 2, "gmm": 3}


def select_bad_dofs(strategy: str, score, p1=0.0, p2=0.0, i1=0, i2=0) -> np.ndarray:
    """MASSolver's bad-DOF selection (host code of the library) on a score
    vector: "elbow" (|diagonal|), "kmean" (p1 search fraction, p2 jump
    threshold, i1 iterations, i2 expand neighbours) or "gmm" (p1 jump
    threshold, p2 tol, i1 iterations, i2 expand neighbours).  Positions in the
    reference's output order."""
    L = load()
    v = np.ascontiguousarray(score, np.float64)
    out = np.empty(max(len(v), 1), np.int32)
    cnt = C.c_int32(0)
    st = L.lss_op_select_bad_dofs(BAD_DOF_STRATEGIES[strategy], len(v), _p(v, _f64p), p1, p2, i1, i2,
                                  _p(out, _i32p), C.byref(cnt))
    if st:
        raise LssError(st, L.lss_last_error(None).decode())
    return out[:cnt.value].copy()


class Solver:
    """polysolve::linear::Solver for the "GPUHybrid" solver, on one GB300."""

    def __init__(self, params=None):
        self._L = load()
        self._h = C.c_void_p()
        js = params if isinstance(params, str) or params is None else json.dumps(params)
        st = self._L.lss_create(js.encode() if js else None, C.byref(self._h))
        if st:
            raise LssError(st, self._L.lss_last_error(None).decode())
        self._keep = None
        self._n = None

    # --- polysolve static constructor (Solver.cpp:143-173)
    @staticmethod
    def create(params=None):
        return Solver(params)

    def _check(self, st):
        if st:
            raise LssError(st, self._L.lss_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.lss_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- polysolve interface
    def set_parameters(self, params):
        js = params if isinstance(params, str) else json.dumps(params)
        self._check(self._L.lss_set_parameters(self._h, js.encode()))

    def get_info(self) -> dict:
        n = C.c_size_t(0)
        self._L.lss_get_info(self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value + 1)
        self._check(self._L.lss_get_info(self._h, buf, n.value + 1, C.byref(n)))
        return json.loads(buf.value.decode())

    def name(self) -> str:
        buf = C.create_string_buffer(64)
        self._check(self._L.lss_name(self._h, buf, 64))
        return buf.value.decode()

    def analyze_pattern(self, A, precond_num=None):
        n, outer, inner, _ = _csc_arrays(A)
        self._check(self._L.lss_analyze_pattern(self._h, n, len(inner), _p(outer, _i32p), _p(inner, _i32p)))

    def factorize(self, A):
        n, outer, inner, vals = _csc_arrays(A)
        self._check(self._L.lss_factorize(self._h, n, len(vals), _p(outer, _i32p), _p(inner, _i32p),
                                          _p(vals, _f64p)))
        self._keep = (outer, inner)
        self._n = n

    def factorize_device(self, values_ptr: int, stream: int = 0):
        """Refactorize with the values in device memory (same pattern as before)."""
        self._check(self._L.lss_factorize_device(self._h, C.c_void_p(values_ptr), C.c_void_p(stream)))

    def solve_device(self, b_ptr: int, x_ptr: int, stream: int = 0):
        """Solve with b and x (initial guess, overwritten) in device memory."""
        self._check(self._L.lss_solve_device(self._h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), C.c_void_p(stream)))

    def set_problematic_dofs(self, dofs):
        d = np.ascontiguousarray(sorted(set(int(v) for v in dofs)), np.int32)
        self._check(self._L.lss_set_problematic_dofs(self._h, _p(d, _i32p), len(d)))

    def solve(self, b, x=None):
        """Solve A x = b; x (if given) is the initial guess and is overwritten,
        as in Solver::solve (Solver.hpp:120-130).  b may be (n,) or (n, k)."""
        b = np.asarray(b, np.float64)
        if x is None:
            x = np.zeros_like(b)
        if b.ndim == 1:
            bb = np.ascontiguousarray(b)
            xx = np.ascontiguousarray(x, np.float64)
            self._check(self._L.lss_solve(self._h, _p(bb, _f64p), _p(xx, _f64p), 1, len(bb)))
        else:
            bb = np.asfortranarray(b)
            xx = np.asfortranarray(x, np.float64)
            self._check(self._L.lss_solve(self._h, _p(bb, _f64p), _p(xx, _f64p), b.shape[1], b.shape[0]))
        if isinstance(x, np.ndarray) and x is not xx and x.dtype == np.float64 and x.shape == xx.shape:
            x[...] = xx
        return xx

    def solve_transpose(self, g, lam=None):
        g = np.ascontiguousarray(g, np.float64)
        lam = np.zeros_like(g) if lam is None else np.ascontiguousarray(lam, np.float64)
        self._check(self._L.lss_solve_transpose(self._h, _p(g, _f64p), _p(lam, _f64p)))
        return lam

    def grad_A_pattern(self, lam, x):
        lam = np.ascontiguousarray(lam, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        out = np.empty(len(self._keep[1]))
        self._check(self._L.lss_grad_A_pattern(self._h, _p(lam, _f64p), _p(x, _f64p), _p(out, _f64p)))
        return out

    def grad_params_device(self, lam_ptr, x_ptr, n_params, rowptr_ptr, cols_ptr, vals_ptr, out_ptr, stream=0):
        self._check(self._L.lss_grad_params_device(self._h, C.c_void_p(lam_ptr), C.c_void_p(x_ptr), n_params,
                                                   C.c_void_p(rowptr_ptr), C.c_void_p(cols_ptr),
                                                   C.c_void_p(vals_ptr), C.c_void_p(out_ptr), C.c_void_p(stream)))

    # --- inspection (parity tests)
    def selected_dofs(self) -> np.ndarray:
        c = C.c_int32(0)
        self._check(self._L.lss_selected_dofs(self._h, None, 0, C.byref(c)))
        out = np.empty(max(c.value, 1), np.int32)
        self._check(self._L.lss_selected_dofs(self._h, _p(out, _i32p), len(out), C.byref(c)))
        return out[:c.value].copy()

    def gmm_selection(self) -> np.ndarray:
        c = C.c_int32(0)
        self._check(self._L.lss_gmm_selection(self._h, None, 0, C.byref(c)))
        out = np.empty(max(c.value, 1), np.int32)
        self._check(self._L.lss_gmm_selection(self._h, _p(out, _i32p), len(out), C.byref(c)))
        return out[:c.value].copy()

    def subdomains(self):
        ns, nd = C.c_int32(0), C.c_int32(0)
        self._check(self._L.lss_subdomains(self._h, None, 0, None, 0, C.byref(ns), C.byref(nd)))
        offs = np.empty(ns.value + 1, np.int32)
        dofs = np.empty(max(nd.value, 1), np.int32)
        self._check(self._L.lss_subdomains(self._h, _p(offs, _i32p), len(offs), _p(dofs, _i32p), len(dofs),
                                           C.byref(ns), C.byref(nd)))
        return [dofs[offs[i]:offs[i + 1]].copy() for i in range(ns.value)]

    def partition(self):
        npart = C.c_int32(0)
        self._check(self._L.lss_partition(self._h, None, 0, None, 0, C.byref(npart)))
        nb = self._n // self.get_info().get("block_size", 1)
        perm = np.empty(nb, np.int32)
        offs = np.empty(npart.value + 1, np.int32)
        self._check(self._L.lss_partition(self._h, _p(perm, _i32p), nb, _p(offs, _i32p), len(offs),
                                          C.byref(npart)))
        return perm, offs

    def spmv(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty_like(x)
        self._check(self._L.lss_op_spmv(self._h, _p(x, _f64p), _p(y, _f64p)))
        return y

    def row_scores(self):
        """(|diagonal|, max |off-diagonal|, l1 norm) per scalar row of the
        permuted operator (partition order)."""
        n = self._n
        d, o, l = np.empty(n), np.empty(n), np.empty(n)
        self._check(self._L.lss_op_row_scores(self._h, _p(d, _f64p), _p(o, _f64p), _p(l, _f64p)))
        return d, o, l

    def spmv_outer(self, x):
        """A x with the PCG's own product (FP64 or double-float, gb300.outer_spmv)."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty_like(x)
        self._check(self._L.lss_op_spmv_outer(self._h, _p(x, _f64p), _p(y, _f64p)))
        return y

    def mas_apply(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.empty_like(r)
        self._check(self._L.lss_op_mas_apply(self._h, _p(r, _f64p), _p(z, _f64p)))
        return z

    def precond(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.empty_like(r)
        self._check(self._L.lss_op_precond(self._h, _p(r, _f64p), _p(z, _f64p)))
        return z

    def time_op(self, kind: int, reps: int = 20):
        ms, by = C.c_double(0), C.c_double(0)
        self._check(self._L.lss_op_time(self._h, kind, reps, C.byref(ms), C.byref(by)))
        return ms.value, by.value
