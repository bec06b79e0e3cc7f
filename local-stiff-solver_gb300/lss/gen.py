"""Seeded synthetic systems with the shapes of the benchmark workloads.

All inputs are synthetic: numpy ``Generator(PCG64(seed))`` drives geometry,
materials, right-hand sides and the choice of collapsed triangles / springs.

* ``elasticity_cube``   -- P1-tet linear elasticity on a structured node grid
  (6 tets per hex, Kuhn split), Dirichlet clamp of the z=0 face kept as
  identity rows, optional diagonal penalty springs.  Assembly is native
  (``liblss_gen.so``, built from ``csrc/gen_elasticity.cpp``).
* ``laplacian_delaunay`` -- scalar P1 Laplacian on a Delaunay triangulation
  of uniform points with a fraction of triangles collapsed to a large aspect
  ratio, Dirichlet on the convex hull.
* ``workload_*`` -- the named workloads (sizes in the function names).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import scipy.sparse as sp

from . import _paths


def _gen_lib():
    path = _paths.gen_lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} missing: run lss.build.build() first")
    L = C.CDLL(path)
    f = L.lss_gen_elasticity_tet
    f.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_double), C.c_double, C.c_int32,
                  C.c_int32, C.POINTER(C.c_int32), C.c_double, C.c_int64, C.POINTER(C.c_int32),
                  C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    f.restype = C.c_int64
    return L


def tet_centroids(nx, ny, nz):
    """Centroids (6 * cells, 3) of the Kuhn tets, in the same order as the assembler."""
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    h = np.array([1.0 / (nx - 1), 1.0 / (ny - 1), 1.0 / (nz - 1)])
    ck, cj, ci = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    origin = np.stack([ci.ravel(), cj.ravel(), ck.ravel()], axis=1).astype(np.float64)
    out = np.empty((origin.shape[0], 6, 3))
    for p, perm in enumerate(perms):
        v = np.zeros(3)
        acc = v.copy()
        for a in range(3):
            v = v.copy()
            v[perm[a]] += 1
            acc += v
        # vertices: 0, e_p0, e_p0+e_p1, (1,1,1) -> sum of offsets / 4
        out[:, p, :] = (origin + (acc + 0.0) / 4.0) * h
    return out.reshape(-1, 3)


def elasticity_cube(nx, ny, nz, E_tet, nu=0.3, clamp_z0=True, spring_nodes=None, spring_k=1e8):
    """CSR (== CSC) matrix of the assembled system, shape (3N, 3N)."""
    N = nx * ny * nz
    E_tet = np.ascontiguousarray(E_tet, np.float64)
    assert E_tet.shape == (6 * (nx - 1) * (ny - 1) * (nz - 1),)
    sn = np.ascontiguousarray(spring_nodes if spring_nodes is not None else [], np.int32)
    cap = 135 * N
    outer = np.empty(3 * N + 1, np.int32)
    inner = np.empty(cap, np.int32)
    vals = np.empty(cap, np.float64)
    nnz = _gen_lib().lss_gen_elasticity_tet(
        nx, ny, nz, E_tet.ctypes.data_as(C.POINTER(C.c_double)), nu, int(bool(clamp_z0)), len(sn),
        sn.ctypes.data_as(C.POINTER(C.c_int32)), spring_k, cap,
        outer.ctypes.data_as(C.POINTER(C.c_int32)), inner.ctypes.data_as(C.POINTER(C.c_int32)),
        vals.ctypes.data_as(C.POINTER(C.c_double)))
    if nnz < 0:
        raise RuntimeError(f"elasticity assembly failed ({nnz})")
    return sp.csr_matrix((vals[:nnz], inner[:nnz], outer), shape=(3 * N, 3 * N))


def sphere_inclusion_E(nx, ny, nz, rng, radius=0.15, E_in=1e6, E_out=1.0):
    """E per tet: E_in for tets whose centroid lies in a sphere of the given
    radius with a seeded centre in [0.25, 0.75]^3, E_out elsewhere."""
    centre = rng.uniform(0.25, 0.75, size=3)
    c = tet_centroids(nx, ny, nz)
    inside = ((c - centre) ** 2).sum(axis=1) < radius * radius
    return np.where(inside, E_in, E_out), centre


def laplacian_delaunay(npts, rng, collapse_frac=0.02, aspect=1e4):
    """Scalar P1 Laplacian on a Delaunay triangulation of npts uniform points in
    the unit square.  collapse_frac of the triangles (seeded) get one interior
    vertex moved toward the opposite edge until base/height == aspect; a move
    that would invert any triangle of that vertex's star is rejected.
    Dirichlet (identity rows) on convex-hull vertices.  Returns (A, info)."""
    from scipy.spatial import Delaunay
    pts = rng.uniform(0.0, 1.0, size=(npts, 2))
    tri = Delaunay(pts)
    T = tri.simplices.astype(np.int64)
    hull = np.unique(tri.convex_hull.ravel())
    on_hull = np.zeros(npts, bool)
    on_hull[hull] = True

    def orient(t):
        p = pts[T[t]]
        return (p[..., 1, 0] - p[..., 0, 0]) * (p[..., 2, 1] - p[..., 0, 1]) - \
               (p[..., 1, 1] - p[..., 0, 1]) * (p[..., 2, 0] - p[..., 0, 0])

    sign0 = np.sign(orient(np.arange(len(T))))
    # vertex -> incident triangles
    order = np.argsort(T.ravel(), kind="stable")
    vstart = np.searchsorted(T.ravel()[order], np.arange(npts + 1))
    inc = order // 3

    ncol = int(round(collapse_frac * len(T)))
    chosen = rng.choice(len(T), size=ncol, replace=False)
    which = rng.integers(0, 3, size=ncol)
    moved = rejected = 0
    for t, w in zip(chosen, which):
        verts = T[t]
        cand = [verts[(w + s) % 3] for s in range(3) if not on_hull[verts[(w + s) % 3]]]
        if not cand:
            rejected += 1
            continue
        v = cand[0]
        a, b = [x for x in verts if x != v]
        pa, pb, pv = pts[a], pts[b], pts[v]
        e = pb - pa
        L = np.hypot(e[0], e[1])
        foot = pa + e * np.dot(pv - pa, e) / (L * L)
        hcur = np.hypot(*(pv - foot))
        htarget = L / aspect
        if hcur <= htarget:
            continue
        newp = foot + (pv - foot) * (htarget / hcur)
        star = inc[vstart[v]:vstart[v + 1]]
        old = pts[v].copy()
        pts[v] = newp
        if np.any(np.sign(orient(star)) != sign0[star]):
            pts[v] = old
            rejected += 1
        else:
            moved += 1

    p = pts[T]  # (nt, 3, 2)
    x, y = p[..., 0], p[..., 1]
    bcoef = np.stack([y[:, 1] - y[:, 2], y[:, 2] - y[:, 0], y[:, 0] - y[:, 1]], axis=1)
    ccoef = np.stack([x[:, 2] - x[:, 1], x[:, 0] - x[:, 2], x[:, 1] - x[:, 0]], axis=1)
    area2 = np.abs(x[:, 1] * y[:, 2] - x[:, 2] * y[:, 1] - x[:, 0] * y[:, 2] + x[:, 2] * y[:, 0]
                   + x[:, 0] * y[:, 1] - x[:, 1] * y[:, 0])
    Ke = (bcoef[:, :, None] * bcoef[:, None, :] + ccoef[:, :, None] * ccoef[:, None, :]) / \
        (2.0 * area2)[:, None, None]
    rows = np.repeat(T, 3, axis=1).ravel()
    cols = np.tile(T, (1, 3)).ravel()
    vals = Ke.ravel()
    keep = ~(on_hull[rows] | on_hull[cols])
    rows = np.concatenate([rows[keep], hull])
    cols = np.concatenate([cols[keep], hull])
    vals = np.concatenate([vals[keep], np.ones(len(hull))])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(npts, npts))
    A.sum_duplicates()
    A.eliminate_zeros()
    A.sort_indices()
    return A, {"triangles": int(len(T)), "collapsed": moved, "rejected": rejected,
               "hull_vertices": int(len(hull))}


# ---------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------

def workload_elasticity_inclusion(seed=0, nodes=20, radius=0.15, E_ratio=1e6, rhs="uniform",
                                  nrhs=1):
    """Cube of nodes^3 grid nodes, stiff spherical inclusion, clamp z=0.
    nodes=20 gives the 24,000-DOF plain small system."""
    rng = np.random.Generator(np.random.PCG64(seed))
    E, centre = sphere_inclusion_E(nodes, nodes, nodes, rng, radius=radius, E_in=E_ratio)
    A = elasticity_cube(nodes, nodes, nodes, E)
    n = A.shape[0]
    b = rng.uniform(-1.0, 1.0, size=(n, nrhs)) if rhs == "uniform" else rng.standard_normal((n, nrhs))
    return A, (b[:, 0] if nrhs == 1 else b), {"centre": centre.tolist(), "seed": seed,
                                              "nodes": nodes, "block_size": 3}


def workload_delaunay_laplacian(seed=0, npts=1_000_000, collapse_frac=0.02, aspect=1e4):
    """2D Delaunay P1 Laplacian with collapsed triangles (1,000,000 points by default)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    A, info = laplacian_delaunay(npts, rng, collapse_frac, aspect)
    b = rng.standard_normal(A.shape[0])
    info.update({"seed": seed, "npts": npts, "block_size": 1})
    return A, b, info


def workload_elasticity_lognormal(seed=0, nodes=100, spring_frac=0.01, spring_k=1e8):
    """nodes^3 grid, E ~ lognormal(0, 1) per tet, penalty springs on a seeded
    fraction of the top-face nodes, clamp z=0 (100 nodes: 3.0M DOFs)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ntet = 6 * (nodes - 1) ** 3
    E = rng.lognormal(0.0, 1.0, size=ntet)
    top = np.arange(nodes * nodes, dtype=np.int64) + (nodes - 1) * nodes * nodes
    ns = max(1, int(round(spring_frac * len(top))))
    springs = np.sort(rng.choice(top, size=ns, replace=False)).astype(np.int32)
    A = elasticity_cube(nodes, nodes, nodes, E, spring_nodes=springs, spring_k=spring_k)
    b = rng.standard_normal(A.shape[0])
    return A, b, {"seed": seed, "nodes": nodes, "springs": int(ns), "block_size": 3}


def workload_batched(seed=0, count=64, dof_lo=5_000, dof_hi=200_000, nrhs=16, radius=0.15):
    """`count` elasticity cubes with DOFs ~ U[dof_lo, dof_hi], each with a seeded
    stiff inclusion of E ratio log-uniform in [1e3, 1e7] and nrhs N(0,1) RHS."""
    rng = np.random.Generator(np.random.PCG64(seed))
    systems = []
    for s in range(count):
        dofs = rng.uniform(dof_lo, dof_hi)
        m = max(3, int(round((dofs / 3.0) ** (1.0 / 3.0))))
        ratio = 10.0 ** rng.uniform(3.0, 7.0)
        E, centre = sphere_inclusion_E(m, m, m, rng, radius=radius, E_in=ratio)
        A = elasticity_cube(m, m, m, E)
        B = rng.standard_normal((A.shape[0], nrhs))
        systems.append((A, B, {"nodes": m, "E_ratio": ratio}))
    return systems


# ---------------------------------------------------------------------------
# parametric elasticity: A(theta) = M theta + c (differentiation workload)
# ---------------------------------------------------------------------------

_KUHN = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def _tet_offsets(p):
    v = [np.zeros(3, int)]
    for a in range(3):
        w = v[-1].copy()
        w[_KUHN[p][a]] += 1
        v.append(w)
    return np.array(v)  # 4 x 3 vertex offsets (in cells)


def _tet_stiffness_ref(p, h, nu):
    """12x12 P1-tet stiffness of Kuhn tet p for E = 1 (same formulas as the
    native assembler)."""
    X = _tet_offsets(p) * h
    J = (X[1:] - X[0]).T
    inv = np.linalg.inv(J)
    g = np.zeros((4, 3))
    g[1:] = inv
    g[0] = -g[1:].sum(axis=0)
    vol = abs(np.linalg.det(J)) / 6.0
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1.0 / (2 * (1 + nu))
    B = np.zeros((6, 12))
    for a in range(4):
        gx, gy, gz = g[a]
        B[0, 3 * a] = gx
        B[1, 3 * a + 1] = gy
        B[2, 3 * a + 2] = gz
        B[3, 3 * a + 1], B[3, 3 * a + 2] = gz, gy
        B[4, 3 * a], B[4, 3 * a + 2] = gz, gx
        B[5, 3 * a], B[5, 3 * a + 1] = gy, gx
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] += 2 * mu
    D[np.arange(3, 6), np.arange(3, 6)] = mu
    return vol * B.T @ D @ B


def elasticity_parametric(nodes, nu=0.3, clamp_z0=True):
    """Structure of A(theta) = sum_e theta_e K_e + c for the Kuhn-tet cube with
    one Young's modulus per tet.  Returns (pattern, M, c): pattern is a CSR
    matrix (values = A(1)), M the (nnz x ntets) map with A.values = M @ theta + c,
    c the identity entries of clamped DOFs.  No entry is pruned, so the pattern
    holds for every theta."""
    n = nodes
    N = n ** 3
    h = np.full(3, 1.0 / (n - 1))
    ck, cj, ci = np.meshgrid(np.arange(n - 1), np.arange(n - 1), np.arange(n - 1), indexing="ij")
    origin = np.stack([ci.ravel(), cj.ravel(), ck.ravel()], axis=1)
    ncell = origin.shape[0]
    rows, cols, vals, tet = [], [], [], []
    clamped = np.zeros(N, bool)
    if clamp_z0:
        clamped[: n * n] = True
    for p in range(6):
        K = _tet_stiffness_ref(p, h, nu)
        off = _tet_offsets(p)
        nodes_p = origin[:, None, :] + off[None, :, :]  # ncell x 4 x 3
        nid = nodes_p[..., 0] + n * (nodes_p[..., 1] + n * nodes_p[..., 2])
        dof = (3 * nid[:, :, None] + np.arange(3)[None, None, :]).reshape(ncell, 12)
        r = np.repeat(dof, 12, axis=1)
        c_ = np.tile(dof, (1, 12))
        v = np.broadcast_to(K.ravel(), (ncell, 144))
        t = np.repeat((np.arange(ncell) * 6 + p)[:, None], 144, axis=1)
        keep = (v != 0) & ~clamped[r // 3] & ~clamped[c_ // 3]
        rows.append(r[keep]); cols.append(c_[keep]); vals.append(v[keep]); tet.append(t[keep])
    rows = np.concatenate(rows); cols = np.concatenate(cols); vals = np.concatenate(vals); tet = np.concatenate(tet)
    cd = np.nonzero(np.repeat(clamped, 3))[0]
    keys = np.concatenate([rows.astype(np.int64) * (3 * N) + cols, cd.astype(np.int64) * (3 * N) + cd])
    ukeys, inv = np.unique(keys, return_inverse=True)
    nnz = len(ukeys)
    prow = (ukeys // (3 * N)).astype(np.int32)
    pcol = (ukeys % (3 * N)).astype(np.int32)
    ntet = 6 * ncell
    M = sp.csr_matrix((vals, (inv[: len(vals)], tet)), shape=(nnz, ntet))
    c = np.zeros(nnz)
    c[inv[len(vals):]] = 1.0
    indptr = np.zeros(3 * N + 1, np.int64)
    np.add.at(indptr, prow + 1, 1)
    indptr = np.cumsum(indptr)
    pattern = sp.csr_matrix((M @ np.ones(ntet) + c, pcol, indptr), shape=(3 * N, 3 * N))
    return pattern, M, c
