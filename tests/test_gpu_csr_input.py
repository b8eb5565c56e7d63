"""Matrices that arrive as CSR (cf_matrix_create_csr), e.g. read from the
reference's file formats: in the reference summation order every solver
reproduces the oracle bit for bit, as it does for the same matrix built
from LDU; the A^T the library builds for BiCG from the CSR arrays equals
the reference's Transpose."""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["CG", "BiCG", "Jacobi", "MRS"])
def test_csr_matrix_from_file_solves_bit_exact(ctx, ref_grid, tmp_path, name):
    kind = O.SOLVER_NAMES[name]
    L = O.grid_convdiff(10, 9, 8, 3)[0] if name == "BiCG" else O.grid_lognormal(10, 9, 8, 2)
    A = O.ldu2csr(L)
    path = str(tmp_path / "A.bin")
    cf.save_csr(path, A.n, A.n, A.row_offsets, A.cols, A.vals)
    n, _, ro, ci, va = cf.read_csr(path)
    M = cf.CsrMatrix(n, ro, ci, va, context=ctx)
    assert M.symmetric() == (name != "BiCG")
    b = O.uniform(3, n)
    want = O.plugin_solve(kind, L, b, np.zeros(n), 1e-8, 5000, grid=ref_grid)
    psi = np.zeros(n)
    perf = cf.New("p", M, {"solver": "cuFoam" + name, "tolerance": 1e-8, "maxIter": 5000,
                           "reduction": "reference"}).solve(psi, b, history=5001)
    assert perf.n_iterations == want.n_iterations
    assert perf.history.tobytes() == want.history.tobytes()
    assert psi.tobytes() == want.psi.tobytes()


def test_csr_matrix_rejects_ldu_only_calls(ctx):
    A = O.ldu2csr(O.grid_const(8, 8, 1))
    M = cf.CsrMatrix(A.n, A.row_offsets, A.cols, A.vals, context=ctx)
    with pytest.raises(NotImplementedError):
        M.update_values(np.ones(A.n), np.ones(1), np.ones(1))
    bad = A.cols.copy()
    bad[3] = A.n + 5
    with pytest.raises(cf.CufoamError):
        cf.CsrMatrix(A.n, A.row_offsets, bad, A.vals, context=ctx)
    # fast SpMV through SELL-32 and CSR agree with the reference-order one to rounding
    x = O.uniform(1, A.n)
    y = M.spmv(x, row_order="fast")
    assert np.allclose(y, O.ref_spmv(A, x), rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("fmt", ["auto", "csr", "sell"])
def test_csr_values_update_on_the_same_pattern(ctx, ref_grid, fmt):
    """cf_matrix_update_csr_values: new values on a CSR-built matrix reach
    every copy the solvers read (CSR, SELL-32 values, the diagonal and its
    inverse, A^T): reference-order Jacobi and BiCG reproduce the oracle on
    the new matrix bit for bit."""
    L1 = O.grid_convdiff(10, 9, 8, 3)[0]
    L2 = O.grid_convdiff(10, 9, 8, 7, 2.0)[0]
    A1, A2 = O.ldu2csr(L1), O.ldu2csr(L2)
    assert np.array_equal(A1.cols, A2.cols) and not np.array_equal(A1.vals, A2.vals)
    M = cf.CsrMatrix(A1.n, A1.row_offsets, A1.cols, A1.vals, context=ctx)
    M.set_format(fmt)
    b = O.uniform(3, A1.n)
    for L, A in ((L1, A1), (L2, A2)):
        if A is A2:
            M.update_csr_values(A2.vals)
        for name in ("Jacobi", "BiCG"):
            kind = O.SOLVER_NAMES[name]
            want = O.plugin_solve(kind, L, b, np.zeros(A.n), 1e-8, 5000, grid=ref_grid)
            psi = np.zeros(A.n)
            perf = cf.New("p", M, {"solver": "cuFoam" + name, "tolerance": 1e-8, "maxIter": 5000,
                                   "reduction": "reference"}).solve(psi, b, history=5001)
            assert perf.n_iterations == want.n_iterations, (name, A is A2)
            assert psi.tobytes() == want.psi.tobytes(), (name, A is A2)


def test_csr_values_update_rejects_ldu_matrices(ctx):
    L = O.grid_const(8, 8, 1)
    M = cf.LduMatrix.from_ldu(L, ctx)
    from cufoam_gb300 import _capi
    lib = _capi.load()
    v = np.ones(M.shape()[2])
    assert lib.cf_matrix_update_csr_values(M._h, v.ctypes.data, _capi.CF_MEM_HOST) == _capi.CF_UNSUPPORTED
