"""Differentiable sparse solve x = A(theta)^-1 b as a torch.autograd.Function.

A(theta) is linear in the parameters: A.values = M @ theta + c on a fixed
pattern (one Young's modulus per element, say).  Forward: assemble the values
on the GPU (the library's kernel), factorize with them in device memory, solve.  Backward: the
adjoint reuses the same factorized hybrid preconditioner and PCG to solve
A^T lambda = dL/dx (A is SPD), then dL/db = lambda and
dL/dtheta_e = -sum_{ij in e} M_(ij),e lambda_i x_j, formed by the library's
fused kernel (lss_grad_params_device) without materialising dL/dA.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import Solver


def _stream_handle():
    h = torch.cuda.current_stream().cuda_stream
    if h == 0:  # legacy default stream: the library orders on its own stream
        torch.cuda.synchronize()
    return h


class LinearSystem:
    """Pattern, parameter map and factorised solver of A(theta) = M theta + c."""

    def __init__(self, pattern, M, c, params: dict, device=None):
        import scipy.sparse as sp
        self.device = torch.device(device or "cuda")
        self.pattern = pattern.tocsr()
        self.n = self.pattern.shape[0]
        self.solver = Solver.create(params)
        self.solver.analyze_pattern(self.pattern)
        M = sp.csr_matrix(M)
        self.n_params = M.shape[1]
        self.n_values = M.shape[0]
        # M in CSR (rows = stored entries of A): the forward's values = M theta + c
        self.m_rowptr = torch.from_numpy(M.indptr.astype(np.int64)).to(self.device)
        self.m_cols = torch.from_numpy(M.indices.astype(np.int32)).to(self.device)
        self.m_vals = torch.from_numpy(M.data.astype(np.float64)).to(self.device)
        Mt = M.T.tocsr()
        self.mt_rowptr = torch.from_numpy(Mt.indptr.astype(np.int64)).to(self.device)
        self.mt_cols = torch.from_numpy(Mt.indices.astype(np.int32)).to(self.device)
        self.mt_vals = torch.from_numpy(Mt.data.astype(np.float64)).to(self.device)
        self.c = torch.from_numpy(np.asarray(c, np.float64)).to(self.device)

    def values(self, theta):
        """A.values = M theta + c, by the library's kernel (lss_assemble_values_device)."""
        from .solver import LssError, load
        th = theta.contiguous()
        out = torch.empty(self.n_values, dtype=torch.float64, device=self.device)
        L = load()
        st = L.lss_assemble_values_device(self.n_values, self.m_rowptr.data_ptr(), self.m_cols.data_ptr(),
                                          self.m_vals.data_ptr(), th.data_ptr(), self.c.data_ptr(), out.data_ptr(),
                                          _stream_handle())
        if st:
            raise LssError(st, L.lss_last_error(None).decode())
        return out


class LinearSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, b, system: LinearSystem):
        vals = system.values(theta.detach()).contiguous()
        bb = b.detach().contiguous()
        x = torch.zeros_like(bb)
        h = _stream_handle()
        system.solver.factorize_device(vals.data_ptr(), h)
        system.solver.solve_device(bb.data_ptr(), x.data_ptr(), h)
        ctx.system = system
        ctx.save_for_backward(x)
        return x

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        system = ctx.system
        gg = g.contiguous()
        lam = torch.zeros_like(gg)
        h = _stream_handle()
        system.solver.solve_device(gg.data_ptr(), lam.data_ptr(), h)  # A^T lambda = g, A symmetric
        dtheta = torch.empty(system.n_params, dtype=torch.float64, device=x.device)
        system.solver.grad_params_device(lam.data_ptr(), x.data_ptr(), system.n_params,
                                         system.mt_rowptr.data_ptr(), system.mt_cols.data_ptr(),
                                         system.mt_vals.data_ptr(), dtheta.data_ptr(), h)
        return dtheta, lam, None


def solve(theta, b, system: LinearSystem):
    return LinearSolve.apply(theta, b, system)
