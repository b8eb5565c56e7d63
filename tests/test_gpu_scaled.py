"""Fast-order Jacobi, MRJacobi, MRS and JMR run on a cached diagonally
scaled copy of the solved matrix (A D^-1, or D^-1/2 A D^-1/2 for JMR).
These tests cover the copy's life cycle.  A transposed solve scales A^T,
and a solve without transpose afterwards scales A again.  New coefficient
values replace the copy."""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O
from conftest import fast_order_iteration_slack

pytestmark = pytest.mark.gpu


def _matrix(ctx, L):
    return cf.LduMatrix.from_ldu(L, ctx)


def _scaled_true_rel(L, b, psi, nf, jmr):
    r = b - O.ref_spmv(O.ldu2csr(L), psi)
    if jmr:  # JMR stops on the D^-1/2-scaled residual
        r = r / np.sqrt(L.diag)
    return np.linalg.norm(r) / nf


@pytest.mark.parametrize("fmt", ["sell", "csr"])
@pytest.mark.parametrize("name", ["Jacobi", "MRJacobi", "MRS", "JMR"])
def test_scaled_matrix_solvers_transpose_and_value_update(ctx, name, fmt):
    """The fast-order Jacobi and MR family run on a cached scaled copy of
    the solved matrix (A D^-1 or D^-1/2 A D^-1/2): a transposed solve scales
    A^T, and new coefficient values replace the cached copy."""
    kind = O.SOLVER_NAMES[name]
    L, _ = O.grid_convdiff(14, 12, 10, 9, 4.0)
    b = O.uniform(5, L.n)
    tol, maxit = 1e-10, 200000
    M = _matrix(ctx, L)
    M.set_format(fmt)
    jmr = name == "JMR"
    for transpose in (False, True, False):
        Ls = L.transposed() if transpose else L
        want = O.plugin_solve(kind, Ls, b, np.zeros(L.n), tol, maxit)
        psi = np.zeros(L.n)
        perf = cf._TABLE["cuFoam" + name]("p", M, {"tolerance": tol, "maxIter": maxit}).solve(
            psi, b, transpose=transpose)
        assert M.format()[0] == fmt
        assert perf.converged, (transpose, perf.status_name)
        assert abs(perf.n_iterations - want.n_iterations) <= fast_order_iteration_slack(want.n_iterations)
        assert _scaled_true_rel(Ls, b, psi, perf.norm_factor, jmr) <= 1.5 * tol
        assert np.linalg.norm(psi - want.psi) <= 1e-6 * np.linalg.norm(want.psi)
    # new values (a stronger diagonal): the next solve must use them
    L2 = O.LDU(L.n, L.diag * 1.5, L.lower.copy(), L.upper.copy(), L.lower_addr, L.upper_addr)
    M.update_values(L2.diag, L2.lower, L2.upper)
    want = O.plugin_solve(kind, L2, b, np.zeros(L.n), tol, maxit)
    psi = np.zeros(L.n)
    perf = cf._TABLE["cuFoam" + name]("p", M, {"tolerance": tol, "maxIter": maxit}).solve(psi, b)
    assert perf.converged
    assert abs(perf.n_iterations - want.n_iterations) <= fast_order_iteration_slack(want.n_iterations)
    assert _scaled_true_rel(L2, b, psi, perf.norm_factor, jmr) <= 1.5 * tol
    assert np.linalg.norm(psi - want.psi) <= 1e-6 * np.linalg.norm(want.psi)
