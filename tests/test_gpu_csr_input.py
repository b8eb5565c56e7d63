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
