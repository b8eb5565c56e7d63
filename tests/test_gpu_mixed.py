"""Mixed precision (FP32 inner solve, FP64 iterative refinement): every
result must reach the FP64 tolerance on the true residual, and its error
against the FP64 oracle solution is stated and bounded."""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O

pytestmark = pytest.mark.gpu


def _true_rel(L, b, x, nf, scaled=False):
    A = O.ldu2csr(L)
    if not scaled:
        return O.true_residual_norm(A, b, x) / nf
    # JMR's residual: D^-1/2 (b - A x)
    r = b - O.ref_spmv(A, x)
    return np.linalg.norm(r / np.sqrt(np.asarray(L.diag, np.float64))) / nf


@pytest.mark.parametrize("name,make", [
    ("BiCG", lambda: O.grid_convdiff(32, 30, 28, 4, 10.0)[0]),
    ("MR", lambda: O.grid_convdiff(20, 18, 16, 5, 10.0)[0]),
    ("MRJacobi", lambda: O.grid_convdiff(20, 18, 16, 5, 10.0)[0]),
    ("MRS", lambda: O.grid_convdiff(20, 18, 16, 5, 10.0)[0]),
    ("JMR", lambda: O.grid_convdiff(20, 18, 16, 5, 10.0)[0]),
    ("CG", lambda: O.grid_lognormal(32, 30, 28, 6)),
])
def test_mixed_reaches_fp64_tolerance(ctx, name, make):
    L = make()
    b = O.uniform(7, L.n)
    tol = 1e-10
    M = cf.LduMatrix.from_ldu(L, ctx)
    psi = np.zeros(L.n)
    perf = cf._TABLE["cuFoam" + name]("p", M, {"tolerance": tol, "maxIter": 200000,
                                              "precision": "mixed"}).solve(psi, b, history=64)
    assert perf.status == 0, perf.status_name
    assert perf.n_outer >= 2
    assert perf.final_residual <= tol
    true_rel = _true_rel(L, b, psi, perf.norm_factor, scaled=name == "JMR")
    assert true_rel <= tol
    # error against the FP64 oracle solution at the same tolerance
    want = O.plugin_solve(O.SOLVER_NAMES[name], L, b, np.zeros(L.n), tol, 200000)
    err = np.linalg.norm(psi - want.psi) / np.linalg.norm(want.psi)
    assert err < 1e-6, err
    # history: FP64 residual per refinement sweep, decreasing
    h = perf.history
    assert h.shape[0] == perf.n_outer + 1
    assert np.all(np.diff(h) < 0)


def test_mixed_unsupported_solvers_are_refused(ctx):
    L = O.grid_lognormal(8, 8, 8, 1)
    M = cf.LduMatrix.from_ldu(L, ctx)
    with pytest.raises(cf.CufoamError) as e:
        cf.cuFoamJacobi("p", M, {"precision": "mixed"}).solve(np.zeros(L.n), np.ones(L.n))
    assert e.value.status == 8


def test_mixed_respects_max_iter(ctx):
    L = O.grid_lognormal(24, 24, 24, 2)
    b = O.uniform(3, L.n)
    M = cf.LduMatrix.from_ldu(L, ctx)
    perf = cf.cuFoamCG("p", M, {"tolerance": 1e-12, "maxIter": 30,
                                "precision": "mixed"}).solve(np.zeros(L.n), b)
    assert perf.n_iterations <= 30
    assert perf.status == 1


@pytest.mark.parametrize("fmt", ["sell8", "sell", "csr"])
@pytest.mark.parametrize("name", ["MRJacobi", "JMR"])
@pytest.mark.parametrize("transpose", [False, True])
def test_mixed_mr_family_formats_and_transpose(ctx, fmt, name, transpose):
    # the FP32 sweep of the preconditioned MR solvers runs MR on a scaled
    # copy of the solved matrix (A or A^T), built from SELL-32 or CSR values
    L, _ = O.grid_convdiff(14, 12, 10, 9, 4.0)
    b = O.uniform(5, L.n)
    tol = 1e-10
    M = cf.LduMatrix.from_ldu(L, ctx)
    M.set_format(fmt)
    psi = np.zeros(L.n)
    perf = cf._TABLE["cuFoam" + name]("p", M, {"tolerance": tol, "maxIter": 200000,
                                              "precision": "mixed"}).solve(psi, b, transpose=transpose)
    assert M.format()[0] == fmt
    assert perf.status == 0, perf.status_name
    Ls = L.transposed() if transpose else L
    assert _true_rel(Ls, b, psi, perf.norm_factor, scaled=name == "JMR") <= tol
    want = O.plugin_solve(O.SOLVER_NAMES[name], Ls, b, np.zeros(L.n), tol, 200000)
    assert np.linalg.norm(psi - want.psi) / np.linalg.norm(want.psi) < 1e-6


def test_mixed_rollback_shortens_the_retry(ctx):
    """A refinement sweep that raises the FP64 residual is undone and retried
    with half as many FP32 steps as the sweep just undone, so a mixed solve
    that cannot make progress stops after a few short retries instead of
    repeating the same deterministic sweep.  Here the FP32 copy of the
    matrix overflows (a diagonal of 1e39 is inf in FP32): the first sweep
    ends non-finite after one step and its retry would have zero steps."""
    L = O.grid_const(16, 16, 1)
    L = O.LDU(L.n, np.full(L.n, 1e39), L.lower, L.upper, L.lower_addr, L.upper_addr)
    b = O.uniform(3, L.n)
    M = cf.LduMatrix.from_ldu(L, ctx)
    psi = np.zeros(L.n)
    perf = cf.cuFoamMR("p", M, {"tolerance": 1e-10, "maxIter": 10000,
                                "precision": "mixed"}).solve(psi, b)
    assert perf.status == 1, perf.status_name          # not converged
    assert perf.n_outer == 1 and perf.n_iterations == 1
    assert np.all(psi == 0.0)                           # the sweep was undone


def test_mixed_bicg_inner_breakdown_is_reported(ctx):
    """The FP32 inner solver of mixed BiCG breaks down before its first step
    when (r^, A r^) = 0, as for a skew-symmetric matrix: the solve stops
    with CF_BREAKDOWN (a retry would repeat the same breakdown)."""
    L = O.LDU(2, np.zeros(2), np.array([-1.0]), np.array([1.0]),
              np.array([0], np.int32), np.array([1], np.int32))
    M = cf.LduMatrix.from_ldu(L, ctx)
    psi = np.zeros(2)
    perf = cf.cuFoamBiCG("p", M, {"tolerance": 1e-12, "maxIter": 100,
                                  "precision": "mixed"}).solve(psi, np.array([1.0, 2.0]))
    assert perf.status == 2, perf.status_name
    assert perf.n_iterations == 0 and perf.n_outer == 1
    assert np.all(psi == 0.0)
