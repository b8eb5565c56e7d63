"""Coupled interfaces through the OpenFOAM plugin layer (the reference
ignores them): a cyclic patch pair is folded into the device matrix as the
entries (faceCell, neighbour faceCell) = -interfaceBouCoeffs appended to
each row (OpenFOAM's interface update, result -= coeffs * psi of the
neighbour patch); the solve must equal the oracle's on that merged matrix
(bit for bit in the reference summation order) and solve the periodic
problem; processor interfaces outside a parallel run are refused
(decomposed runs: test_gpu_decomposed.py)."""
import numpy as np
import pytest

import oracle as O
from cufoam_gb300.plugin import FoamError, coupled_builds, foam_solve

pytestmark = pytest.mark.gpu


def periodic_x(L, nx, ny, nz=1):
    """Cells at x = 0 and x = nx-1 of every (y, z) line: the cyclic pair."""
    fa = np.array([nx * (j + ny * k) for k in range(nz) for j in range(ny)], np.int32)
    return fa, fa + (nx - 1)


def merged_csr(L, fa, fb, ca, cb):
    A = O.ldu2csr(L)
    extra = [[] for _ in range(L.n)]
    for f in range(len(fa)):
        extra[fa[f]].append((fb[f], -ca[f]))
    for f in range(len(fb)):
        extra[fb[f]].append((fa[f], -cb[f]))
    ro, cols, vals = [0], [], []
    for i in range(L.n):
        cols += A.cols[A.row_offsets[i]:A.row_offsets[i + 1]].tolist() + [c for c, _ in extra[i]]
        vals += A.vals[A.row_offsets[i]:A.row_offsets[i + 1]].tolist() + [v for _, v in extra[i]]
        ro.append(len(cols))
    return O.CSR(np.array(ro, np.int32), np.array(cols, np.int32), np.array(vals))


def test_cyclic_poisson_bit_exact_in_reference_order(ref_grid):
    nx, ny = 32, 24
    L = O.grid_const(nx, ny, 1)
    fa, fb = periodic_x(L, nx, ny)
    ca = cb = np.ones(len(fa))
    b = O.uniform(5, L.n)
    tol, maxit = 1e-9, 20000
    A = merged_csr(L, fa, fb, ca, cb)
    nf = O.norm_factor(A, b, np.zeros(L.n), ref_grid)
    want = O.solve(O.CG, A, b, np.zeros(L.n), tol * nf, maxit, ref_grid)
    psi = np.zeros(L.n)
    p = foam_solve("cuFoamCG", L, b, psi, tolerance=tol, max_iter=maxit, cyclic=(fa, fb, ca, cb),
                   reduction="reference")
    assert p["nIterations"] == want.n_iterations
    assert psi.tobytes() == want.x.tobytes()
    assert p["finalResidual"] == want.history[-1] / nf
    # and it is the periodic problem: dense check
    D = A.dense()
    assert np.allclose(D, D.T)
    x = np.linalg.solve(D, b)
    assert np.linalg.norm(psi - x) <= 1e-6 * np.linalg.norm(x)


def test_cyclic_matrix_kept_across_solves(ref_grid):
    """A mesh with cyclic patches keeps its coupled matrix between solves,
    as a running case does from one time step to the next: new cell and
    interface coefficients on the same mesh refresh its values without a
    rebuild; another cyclic pairing on the same mesh builds a new one; every
    solve equals the oracle's on its merged matrix bit for bit (reference
    order)."""
    nx, ny = 32, 24
    L = O.grid_const(nx, ny, 1)
    fa, fb = periodic_x(L, nx, ny)
    b = O.uniform(5, L.n)
    tol, maxit = 1e-9, 20000
    before = coupled_builds()
    cases = [(fb, 1.0, 1.0, 1), (fb, 1.5, 0.5, 1), (np.roll(fb, 1), 1.5, 0.5, 2), (fb, 2.0, 0.25, 2)]
    for pair_b, scale, cval, builds in cases:
        Ls = O.LDU(L.n, L.diag * scale, L.lower * scale, L.upper * scale, L.lower_addr, L.upper_addr)
        ca = cb = np.full(len(fa), cval)
        A = merged_csr(Ls, fa, pair_b, ca, cb)
        nf = O.norm_factor(A, b, np.zeros(L.n), ref_grid)
        want = O.solve(O.CG, A, b, np.zeros(L.n), tol * nf, maxit, ref_grid)
        psi = np.zeros(L.n)
        p = foam_solve("cuFoamCG", Ls, b, psi, tolerance=tol, max_iter=maxit, cyclic=(fa, pair_b, ca, cb),
                       reduction="reference", reuse_addressing=2)
        assert p["nIterations"] == want.n_iterations, (scale, cval)
        assert psi.tobytes() == want.x.tobytes(), (scale, cval)
        assert coupled_builds() == before + builds, (scale, cval)


def test_cyclic_nonsymmetric_bicg_fast_order():
    nx, ny, nz = 12, 10, 8
    L, _ = O.grid_convdiff(nx, ny, nz, 4)
    fa, fb = periodic_x(L, nx, ny, nz)
    ca = np.full(len(fa), 1.5)
    cb = np.full(len(fb), 0.5)
    b = O.uniform(6, L.n)
    psi = np.zeros(L.n)
    p = foam_solve("cuFoamBiCG", L, b, psi, tolerance=1e-9, max_iter=20000, cyclic=(fa, fb, ca, cb))
    A = merged_csr(L, fa, fb, ca, cb)
    nf = O.norm_factor(A, b, np.zeros(L.n))
    assert p["converged"]
    assert O.true_residual_norm(A, b, psi) / nf <= 1.5e-9


def test_processor_interface_outside_a_parallel_run_is_refused():
    L = O.grid_const(8, 8, 1)
    with pytest.raises(FoamError, match="outside a parallel run"):
        foam_solve("cuFoamCG", L, O.uniform(1, L.n), np.zeros(L.n), processor_patch=True)
