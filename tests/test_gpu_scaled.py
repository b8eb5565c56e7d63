"""Fast-order Jacobi and JMR run on a cached diagonally scaled copy of the
solved matrix (A D^-1, or D^-1/2 A D^-1/2 for JMR); MRJacobi and MRS
gather z = D^-1 r like the reference.  These tests cover the scaled copy's
life cycle, and the same transposed solves and value updates for all four
solvers.  A transposed solve scales A^T, and a solve without transpose
afterwards scales A again.  New coefficient values replace the copy."""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O
from conftest import assert_fast_order_parity, reference_band

pytestmark = pytest.mark.gpu


def _matrix(ctx, L):
    return cf.LduMatrix.from_ldu(L, ctx)


def _scaled_true_rel(L, b, psi, nf, jmr):
    r = b - O.ref_spmv(O.ldu2csr(L), psi)
    if jmr:  # JMR stops on the D^-1/2-scaled residual
        r = r / np.sqrt(L.diag)
    return np.linalg.norm(r) / nf


@pytest.mark.parametrize("fmt", ["sell8", "sell", "csr"])
@pytest.mark.parametrize("name", ["Jacobi", "MRJacobi", "MRS", "JMR"])
def test_scaled_matrix_solvers_transpose_and_value_update(ctx, name, fmt):
    """Transposed solves and new coefficient values in the fast order:
    iteration counts within the reference's one-ulp band."""
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
        assert_fast_order_parity(perf, want, reference_band(kind, Ls, b, np.zeros(L.n), tol, maxit), tol)
        assert _scaled_true_rel(Ls, b, psi, perf.norm_factor, jmr) <= 1.5 * tol
        assert np.linalg.norm(psi - want.psi) <= 1e-6 * np.linalg.norm(want.psi)
    # new values (a stronger diagonal): the next solve must use them
    L2 = O.LDU(L.n, L.diag * 1.5, L.lower.copy(), L.upper.copy(), L.lower_addr, L.upper_addr)
    M.update_values(L2.diag, L2.lower, L2.upper)
    want = O.plugin_solve(kind, L2, b, np.zeros(L.n), tol, maxit)
    psi = np.zeros(L.n)
    perf = cf._TABLE["cuFoam" + name]("p", M, {"tolerance": tol, "maxIter": maxit}).solve(psi, b)
    assert perf.converged
    assert_fast_order_parity(perf, want, reference_band(kind, L2, b, np.zeros(L.n), tol, maxit), tol)
    assert _scaled_true_rel(L2, b, psi, perf.norm_factor, jmr) <= 1.5 * tol
    assert np.linalg.norm(psi - want.psi) <= 1e-6 * np.linalg.norm(want.psi)
