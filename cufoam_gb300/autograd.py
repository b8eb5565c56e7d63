"""Differentiable LDU solve: ``x = solve(diag, lower, upper, source)`` as a
``torch.autograd.Function``.

Forward: the chosen plugin solver (CG by default) on the GPU.
Backward: the adjoint system A^T lambda = dL/dx solved by the same solver
(``transpose`` solve on A's pattern), then the hand-written scatter kernel
``cf_adjoint_gradients`` forms

    dL/d diag[i]  = -lambda_i x_i
    dL/d upper[f] = -lambda_owner[f] x_neighbour[f]
    dL/d lower[f] = -lambda_neighbour[f] x_owner[f]
    dL/d source   =  lambda

(the sparsity pattern is fixed by the addressing; the reference has no
differentiable path, this is new).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import LduMatrix, _TABLE, default_context


class LduPattern:
    """The fixed addressing of a family of LDU matrices on one device; holds
    the library matrix whose values each forward pass refreshes."""

    def __init__(self, n_cells: int, lower_addr, upper_addr, context=None):
        self.ctx = context or default_context()
        self.n = int(n_cells)
        self.lower_addr = torch.as_tensor(lower_addr, dtype=torch.int32).contiguous()
        self.upper_addr = torch.as_tensor(upper_addr, dtype=torch.int32).contiguous()
        self._matrix = None

    def matrix(self, diag, lower, upper) -> LduMatrix:
        dev = diag.device
        la = self.lower_addr.to(dev)
        ua = self.upper_addr.to(dev)
        if self._matrix is None:
            self._matrix = LduMatrix(self.n, diag, lower, upper, la, ua, context=self.ctx)
        else:
            self._matrix.update_values(diag, lower, upper)
        return self._matrix


class LduSolveFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, diag, lower, upper, source, pattern: LduPattern, controls: dict):
        diag, lower, upper, source = (t.detach().contiguous() for t in (diag, lower, upper, source))
        M = pattern.matrix(diag, lower, upper)
        solver = _TABLE[controls.get("solver", "cuFoamCG")]("x", M, controls)
        x = torch.zeros_like(source)
        perf = solver.solve(x, source)
        if perf.status not in (0,):
            raise RuntimeError(f"forward solve did not converge: {perf.status_name} "
                               f"(final residual {perf.final_residual:.3e})")
        ctx.pattern = pattern
        ctx.controls = dict(controls)
        ctx.save_for_backward(diag, lower, upper, x)
        ctx.last_perf = perf
        return x

    @staticmethod
    def backward(ctx, grad_x):
        diag, lower, upper, x = ctx.saved_tensors
        pattern: LduPattern = ctx.pattern
        M = pattern.matrix(diag, lower, upper)  # values of this forward pass
        controls = dict(ctx.controls)
        controls["transpose"] = 1
        solver = _TABLE[controls.get("solver", "cuFoamCG")]("lambda", M, controls)
        g = grad_x.detach().contiguous()
        lam = torch.zeros_like(g)
        perf = solver.solve(lam, g, transpose=True)
        if perf.status not in (0,):
            raise RuntimeError(f"adjoint solve did not converge: {perf.status_name}")
        d_diag = torch.empty_like(diag)
        d_lower = torch.empty_like(lower)
        d_upper = torch.empty_like(upper)
        torch.cuda.current_stream(diag.device).synchronize()
        M.ctx.check(M._lib.cf_adjoint_gradients(M.handle, lam.data_ptr(), x.data_ptr(),
                                                d_diag.data_ptr(), d_lower.data_ptr(),
                                                d_upper.data_ptr(), 1),
                    "cf_adjoint_gradients")
        return d_diag, d_lower, d_upper, lam, None, None


def ldu_solve(diag, lower, upper, source, pattern: LduPattern, controls: dict | None = None):
    """Differentiable solve of the LDU system; gradients flow to diag, lower,
    upper and source."""
    c = {"solver": "cuFoamCG", "tolerance": 1e-14, "maxIter": 100000}
    c.update(controls or {})
    return LduSolveFunction.apply(diag, lower, upper, source, pattern, c)
