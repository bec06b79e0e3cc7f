"""Adjoint of x = A(theta)^-1 b through the torch.autograd.Function.

* x1e5 stiff inclusion (10^3 nodes, 3,000 DOFs): loss, parameter gradient and right-hand-side gradient
  against an FP64 dense-solve adjoint (1e-6 relative).
* x1e3 stiff inclusion: parameter gradient against finite differences of the
  solver's own loss on 20 random directions (1e-5 relative).  The differences
  use the fourth-order five-point stencil with a relative step of 1e-2: the
  loss carries solve noise of about cond(A) * tol relative, which a 1e-6
  central difference amplifies by 1e6 (about 1e-2 relative at x1e5, even with
  a dense LU solve); the wide stencil keeps noise and truncation error (both
  near 1e-6) below the bound."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(nodes=10, seed=0, stiff=1e5):
    from lss import gen
    pattern, M, c = gen.elasticity_parametric(nodes)
    rng = np.random.default_rng(seed)
    ntet = M.shape[1]
    theta = np.exp(rng.standard_normal(ntet))
    # stiff inclusion around a seeded centre
    cen = gen.tet_centroids(nodes, nodes, nodes)
    centre = rng.uniform(0.3, 0.7, 3)
    theta[((cen - centre) ** 2).sum(1) < 0.2 ** 2] *= stiff
    b = rng.standard_normal(pattern.shape[0])
    xstar = rng.standard_normal(pattern.shape[0])
    return pattern, M, c, theta, b, xstar


def _dense_grad(pattern, M, c, theta, b, xstar):
    import scipy.sparse as sp
    vals = M @ theta + c
    A = sp.csr_matrix((vals, pattern.indices, pattern.indptr), shape=pattern.shape).toarray()
    x = np.linalg.solve(A, b)
    lam = np.linalg.solve(A.T, x - xstar)
    Ms = M.tocoo()
    rows = np.repeat(np.arange(pattern.shape[0]), np.diff(pattern.indptr))
    colsv = pattern.indices
    contrib = -Ms.data * lam[rows[Ms.row]] * x[colsv[Ms.row]]
    dtheta = np.bincount(Ms.col, weights=contrib, minlength=M.shape[1])
    return 0.5 * np.sum((x - xstar) ** 2), dtheta, lam


PARAMS = {"solver": "GPUHybrid",
          "GPUHybrid": {"block_size": 3, "relative_tolerance": 1e-13, "max_iter": 20000,
                        "decompose_subdomains": False},
          "gb300": {"max_refinements": 4}}


def test_adjoint_matches_dense_adjoint(built):
    import torch
    from lss import autograd as AG
    pattern, M, c, theta, b, xstar = _setup()
    system = AG.LinearSystem(pattern, M, c, PARAMS)
    dev = system.device
    th = torch.tensor(theta, dtype=torch.float64, device=dev, requires_grad=True)
    bt = torch.tensor(b, dtype=torch.float64, device=dev, requires_grad=True)
    xs = torch.tensor(xstar, dtype=torch.float64, device=dev)
    x = AG.solve(th, bt, system)
    L = 0.5 * ((x - xs) ** 2).sum()
    L.backward()
    Ld, gd, lamd = _dense_grad(pattern, M, c, theta, b, xstar)
    assert abs(L.item() - Ld) <= 1e-9 * abs(Ld)
    g = th.grad.cpu().numpy()
    assert np.linalg.norm(g - gd) <= 1e-6 * np.linalg.norm(gd)
    assert np.linalg.norm(bt.grad.cpu().numpy() - lamd) <= 1e-6 * np.linalg.norm(lamd)


def test_adjoint_matches_finite_differences(built):
    import torch
    from lss import autograd as AG
    pattern, M, c, theta, b, xstar = _setup(stiff=1e3)
    system = AG.LinearSystem(pattern, M, c, PARAMS)
    dev = system.device
    th = torch.tensor(theta, dtype=torch.float64, device=dev, requires_grad=True)
    bt = torch.tensor(b, dtype=torch.float64, device=dev)
    xs = torch.tensor(xstar, dtype=torch.float64, device=dev)
    L = 0.5 * ((AG.solve(th, bt, system) - xs) ** 2).sum()
    L.backward()
    g = th.grad.cpu().numpy()

    def loss(t):
        with torch.no_grad():
            xx = AG.solve(torch.tensor(t, dtype=torch.float64, device=dev), bt, system)
            return 0.5 * ((xx - xs) ** 2).sum().item()

    rng = np.random.default_rng(7)
    h = 1e-2
    worst = 0.0
    for _ in range(20):
        d = rng.standard_normal(len(theta)) * theta  # relative perturbation direction
        fd = (-loss(theta + 2 * h * d) + 8 * loss(theta + h * d) - 8 * loss(theta - h * d)
              + loss(theta - 2 * h * d)) / (12 * h)
        an = float(g @ d)
        worst = max(worst, abs(fd - an) / max(abs(an), 1e-30))
    assert worst <= 1e-5, worst
