"""Batched solves (lss_factorize_batched_device + lss_solve_batched_device)
through the C ABI: several elasticity systems of uneven size with stiff
inclusions, several right-hand sides each, solved at once.

* every (system, right-hand side) solution is bit-identical to solving it
  alone with the same solver afterwards (each system runs the single-system
  path on its own stream; the launch shape is fixed so nothing is timed);
* every solve reaches a true relative residual <= 1e-8 and agrees with
  scipy's FP64 sparse direct solve to 1e-6;
* iteration counts are reported per solve; the same solver twice is rejected.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = {"block_size": 3, "relative_tolerance": 1e-8, "gmm_jump_threshold": 10.0, "min_subdomain_size": 4}


def _systems():
    from lss import gen
    out = []
    for A, B, info in gen.workload_batched(seed=3, count=5, dof_lo=2_000, dof_hi=20_000, nrhs=3):
        A = A.tocsc()
        A.sum_duplicates()
        out.append((A, np.asfortranarray(B)))
    return out


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batched_matches_single_solves(precision, built):
    import torch
    import scipy.sparse.linalg as spla
    import lss
    dev = torch.device("cuda", 0)
    systems = _systems()
    solvers, vals, bs, xs = [], [], [], []
    for A, B in systems:
        s = lss.Solver.create({"solver": "GPUHybrid", "GPUHybrid": PARAMS,
                               "gb300": {"precision": precision, "spmv_lanes": 4}})
        s.analyze_pattern(A)
        solvers.append(s)
        vals.append(torch.tensor(A.data, dtype=torch.float64, device=dev))
        bs.append(torch.tensor(B.T.copy(), dtype=torch.float64, device=dev))  # rows = right-hand sides
        xs.append(torch.zeros_like(bs[-1]))
    lss.factorize_batched_device(solvers, [v.data_ptr() for v in vals])
    nrhs = systems[0][1].shape[1]
    its = lss.solve_batched_device(solvers, [b.data_ptr() for b in bs], [x.data_ptr() for x in xs], nrhs)
    torch.cuda.synchronize()
    assert its.shape == (len(systems), nrhs) and (its > 0).all()
    for si, ((A, B), s) in enumerate(zip(systems, solvers)):
        Ar = A.tocsr()
        for k in range(nrhs):
            x = xs[si][k].cpu().numpy()
            b = B[:, k]
            rel = np.linalg.norm(b - Ar @ x) / np.linalg.norm(b)
            assert rel <= 1e-8, (si, k, rel)
            xd = spla.spsolve(A, b)
            assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd), (si, k)
            # the same solve alone with the same solver: bit-identical
            x1 = torch.zeros(A.shape[0], dtype=torch.float64, device=dev)
            s.solve_device(bs[si][k].data_ptr(), x1.data_ptr())
            torch.cuda.synchronize()
            assert torch.equal(x1, xs[si][k]), (si, k)
            assert s.get_info()["num_iterations"] == its[si, k]


def test_batched_rejects_repeated_solver(built):
    import torch
    import lss
    A, B = _systems()[0]
    s = lss.Solver.create({"solver": "GPUHybrid", "GPUHybrid": PARAMS})
    s.factorize(A)
    b = torch.tensor(B[:, 0], dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    with pytest.raises(lss.LssError) as e:
        lss.solve_batched_device([s, s], [b.data_ptr()] * 2, [x.data_ptr()] * 2, 1)
    assert "distinct" in str(e.value)
