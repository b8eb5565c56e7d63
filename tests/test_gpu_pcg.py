"""Jacobi-preconditioned CG (cuFoamPCG; no reference counterpart -- the
reference's roadmap announces preconditioners): checked against a textbook
PCG with z = D^-1 r in numpy FP64 on the same system and stopping rule
(||r||_2 <= tolerance * normFactor): iteration count within the band of
counts textbook PCG takes when one source entry moves by one ulp (widened
by one step plus its width), true residual at the tolerance; on
high-contrast coefficients it needs fewer steps than CG."""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O

pytestmark = pytest.mark.gpu


def numpy_pcg(A, b, tol_abs, max_it):
    import scipy.sparse as sp
    M = sp.csr_matrix((A.vals, A.cols, A.row_offsets), shape=(A.n, A.n))
    dinv = 1.0 / M.diagonal()
    x = np.zeros(A.n)
    r = b.copy()
    z = dinv * r
    p = z.copy()
    rz = r @ z
    k = 0
    while np.linalg.norm(r) > tol_abs and k < max_it:
        q = M @ p
        xi = rz / (p @ q)
        x += xi * p
        r -= xi * q
        k += 1
        z = dinv * r
        rz, rz_old = r @ z, rz
        p = z + (rz / rz_old) * p
    return x, k


@pytest.mark.parametrize("case", ["lognormal", "const"])
def test_pcg_matches_textbook_pcg(ctx, case):
    L = O.grid_lognormal(24, 20, 16, 5) if case == "lognormal" else O.grid_const(20, 18, 16)
    A = O.ldu2csr(L)
    b = O.uniform(3, L.n)
    tol, maxit = 1e-9, 5000
    M = cf.LduMatrix.from_ldu(L, ctx)
    nf = O.norm_factor(A, b, np.zeros(L.n))
    ks = [numpy_pcg(A, b, tol * nf, maxit)[1]]
    rng = np.random.default_rng(11)
    for t in range(8):   # the textbook PCG's own one-ulp band
        bb = b.copy()
        i = int(rng.integers(L.n))
        bb[i] = np.nextafter(bb[i], np.inf if t % 2 == 0 else -np.inf)
        ks.append(numpy_pcg(A, bb, tol * nf, maxit)[1])
    for use_graph in (1, 0):
        psi = np.zeros(L.n)
        perf = cf.cuFoamPCG("p", M, {"tolerance": tol, "maxIter": maxit, "useGraph": use_graph}).solve(psi, b)
        assert perf.converged and perf.final_residual <= tol
        w = max(ks) - min(ks)
        assert min(ks) - 1 - w <= perf.n_iterations <= max(ks) + 1 + w, (perf.n_iterations, ks)
        assert O.true_residual_norm(A, b, psi) / perf.norm_factor <= 1.5 * tol
    if case == "lognormal":
        cg = cf.cuFoamCG("p", M, {"tolerance": tol, "maxIter": maxit}).solve(np.zeros(L.n), b)
        assert perf.n_iterations < cg.n_iterations


def test_pcg_limits(ctx):
    L = O.grid_const(16, 16, 1)
    M = cf.LduMatrix.from_ldu(L, ctx)
    b = O.uniform(1, L.n)
    with pytest.raises(cf.CufoamError) as e:
        cf.cuFoamPCG("p", M, {"reduction": "reference"}).solve(np.zeros(L.n), b)
    assert e.value.status == 8   # unsupported: no reference summation order
    with pytest.raises(cf.CufoamError):
        cf.cuFoamPCG("p", M, {"precision": "mixed"}).solve(np.zeros(L.n), b)
    with pytest.raises(KeyError):
        cf.New("U", _Asym(), {"solver": "cuFoamPCG"})   # symmetric table only


class _Asym:
    def symmetric(self):
        return False


def test_pcg_through_the_openfoam_plugin():
    from cufoam_gb300.plugin import foam_solve
    L = O.grid_lognormal(16, 14, 12, 8)
    A = O.ldu2csr(L)
    b = O.uniform(9, L.n)
    psi = np.zeros(L.n)
    p = foam_solve("cuFoamPCG", L, b, psi, tolerance=1e-8, max_iter=5000)
    assert p["converged"] and p["finalResidual"] <= 1e-8
    assert O.true_residual_norm(A, b, psi) / O.norm_factor(A, b, np.zeros(L.n)) <= 1.5e-8
