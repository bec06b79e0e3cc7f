"""Allocation-free selection entry point (lss_gmm_select_device_noalloc),
called through the C ABI, against the allocating solver path
(lss_gmm_selection): the same selected rows, bit for bit, on two calls in a
row; n = 0; rejection of n beyond LSS_NOALLOC_MAX_ROWS before any device work.

The file name sorts last so that the test also runs after every other GPU test
of the same process (the static scratch is then already resolved and has
served other calls); it needs nothing from them and passes alone too."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOALLOC_MAX_ROWS = 1 << 20


def _workloads():
    from lss import gen
    A1, _, _ = gen.workload_elasticity_inclusion(seed=0, nodes=20)
    A2, _, _ = gen.workload_elasticity_lognormal(seed=0, nodes=16)
    out = []
    for name, A, threshold in [("inclusion_20", A1, 10.0), ("springs_16", A2, 100.0)]:
        A = A.tocsc()
        A.sum_duplicates()  # the canonical layout the solver itself is given
        out.append((name, A, threshold))
    return out


def test_noalloc_selection_matches_solver_twice(built):
    import torch
    import lss
    L = lss.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    for name, A, threshold in _workloads():
        gmm = {"gmm_jump_threshold": threshold, "gmm_tol": 1e-3, "max_gmm_iterations": 20}
        s = lss.Solver.create({"solver": "GPUHybrid", "GPUHybrid": {"block_size": 3, **gmm}})
        s.factorize(A)
        ref = s.gmm_selection()
        assert len(ref) > 0, name
        n, nnz = A.shape[0], A.nnz
        outer = torch.tensor(A.indptr.astype(np.int32), device=dev)
        vals = torch.tensor(A.data, dtype=torch.float64, device=dev)
        sel = torch.empty(n, dtype=torch.int32, device=dev)
        cnt = torch.empty(1, dtype=torch.int32, device=dev)
        for call in range(2):
            with torch.cuda.stream(stream):
                sel.fill_(-1)
                cnt.fill_(-1)
            st = L.lss_gmm_select_device_noalloc(n, nnz, outer.data_ptr(), vals.data_ptr(), threshold,
                                                 gmm["gmm_tol"], gmm["max_gmm_iterations"], sel.data_ptr(),
                                                 cnt.data_ptr(), C.c_void_p(stream.cuda_stream))
            assert st == 0, (name, call, L.lss_last_error(None))
            stream.synchronize()
            k = int(cnt.item())
            assert k == len(ref), (name, call, k, len(ref))
            np.testing.assert_array_equal(sel[:k].cpu().numpy(), ref)


def test_noalloc_empty_and_oversize(built):
    import torch
    import lss
    L = lss.load()
    dev = torch.device("cuda", 0)
    cnt = torch.full((1,), -1, dtype=torch.int32, device=dev)
    st = L.lss_gmm_select_device_noalloc(0, 0, None, None, 100.0, 1e-3, 20, None, cnt.data_ptr(), None)
    assert st == 0, L.lss_last_error(None)
    torch.cuda.synchronize()
    assert int(cnt.item()) == 0
    small = torch.zeros(16, dtype=torch.int32, device=dev)
    vals = torch.zeros(16, dtype=torch.float64, device=dev)
    st = L.lss_gmm_select_device_noalloc(NOALLOC_MAX_ROWS + 1, 16, small.data_ptr(), vals.data_ptr(), 100.0, 1e-3,
                                         20, small.data_ptr(), cnt.data_ptr(), None)
    assert st == 1 and b"allocation-free limit" in L.lss_last_error(None)
    torch.cuda.synchronize()
    assert int(cnt.item()) == 0  # untouched by the rejected call
