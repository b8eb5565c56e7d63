"""The OpenFOAM plugin layer (cuFoamGB300.C) driven like OpenFOAM drives it:
solver selected by name from the symmetric/asymmetric tables, controls from
the solver dictionary, solve(psi, source, cmpt) -> solverPerformance."""
import numpy as np
import pytest

import oracle as O
from cufoam_gb300.plugin import FoamError, foam_solve
from conftest import reference_band


def test_selection_errors_without_device():
    # the run-time table lookup happens before any device work
    L = O.grid_convdiff(4, 4, 3, 1)[0]
    psi = np.zeros(L.n)
    with pytest.raises(FoamError, match="Unknown asymmetric matrix solver cuFoamCG"):
        foam_solve("cuFoamCG", L, np.ones(L.n), psi, symmetric=False)
    with pytest.raises(FoamError, match="Unknown asymmetric matrix solver cuFoamRichardson"):
        foam_solve("cuFoamRichardson", L, np.ones(L.n), psi, symmetric=False)
    S = O.grid_const(4, 4, 1)
    with pytest.raises(FoamError, match="Unknown symmetric matrix solver PBiCGStab"):
        foam_solve("PBiCGStab", S, np.ones(S.n), np.zeros(S.n))


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(O.SOLVER_NAMES))
def test_plugin_matches_oracle_reference_order(name, ref_grid):
    kind = O.SOLVER_NAMES[name]
    L = O.grid_const(64, 64, 1) if kind != O.BICG else O.grid_convdiff(24, 20, 1, 5)[0]
    b = O.uniform(1, L.n)
    tol, maxit = 1e-6, 40000
    want = O.plugin_solve(kind, L, b, np.zeros(L.n), tol, maxit, grid=ref_grid)
    psi = np.zeros(L.n)
    perf = foam_solve("cuFoam" + name, L, b, psi, tolerance=tol, max_iter=maxit,
                      reduction="reference")
    assert perf["nIterations"] == want.n_iterations
    assert perf["initialResidual"] == want.initial_residual
    assert perf["finalResidual"] == want.final_residual
    assert perf["converged"] == (want.final_residual < tol)
    assert psi.tobytes() == want.psi.tobytes()


@pytest.mark.gpu
def test_plugin_reuses_device_matrix_across_components():
    # Ux, Uy, Uz: same lduMatrix, three sources -> same answers as fresh solves
    L = O.grid_lognormal(20, 18, 16, 3)
    outs = []
    for cmpt in range(3):
        b = O.uniform(10 + cmpt, L.n)
        psi = np.zeros(L.n)
        p = foam_solve("cuFoamCG", L, b, psi, tolerance=1e-9, max_iter=5000)
        lo, hi = reference_band(O.CG, L, b, np.zeros(L.n), 1e-9, 5000)
        assert lo - 1 - (hi - lo) <= p["nIterations"] <= hi + 1 + (hi - lo)
        assert p["converged"]
        outs.append(psi)
    assert not np.array_equal(outs[0], outs[1])


@pytest.mark.gpu
def test_plugin_controls_precision_and_reltol():
    L = O.grid_convdiff(24, 22, 20, 7)[0]
    b = O.uniform(2, L.n)
    psi = np.zeros(L.n)
    p = foam_solve("cuFoamBiCG", L, b, psi, tolerance=1e-10, max_iter=100000, precision="mixed")
    assert p["converged"] and p["finalResidual"] <= 1e-10
    A = O.ldu2csr(L)
    nf = O.norm_factor(A, b, np.zeros(L.n))
    assert O.true_residual_norm(A, b, psi) / nf <= 1e-10
    # relTol honoured only on request (the reference ignores it)
    psi = np.zeros(L.n)
    p1 = foam_solve("cuFoamMR", L, b, psi, tolerance=1e-12, rel_tol=1e-2, max_iter=100000)
    psi = np.zeros(L.n)
    p2 = foam_solve("cuFoamMR", L, b, psi, tolerance=1e-12, rel_tol=1e-2, max_iter=100000,
                    useRelTol="true")
    assert p2["nIterations"] < p1["nIterations"]
    assert p2["finalResidual"] <= 1e-2 * p2["initialResidual"] and p2["converged"]


@pytest.mark.gpu
def test_plugin_matrix_cache_is_keyed_on_the_mesh_not_its_memory():
    """A new mesh built in the memory of an old one (same addressing object,
    same list buffers, same sizes, other faces) must not reuse the old
    device matrix; two meshes solved in turn (a multi-region case) both stay
    cached."""
    from cufoam_gb300.plugin import matrix_builds
    LA = O.grid_lognormal(12, 10, 8, 3)
    LB = O.permute_ldu(LA, O.permutation(7, LA.n))       # same sizes, other faces
    assert LB.lower_addr.shape == LA.lower_addr.shape
    assert not (np.array_equal(LB.lower_addr, LA.lower_addr) and np.array_equal(LB.upper_addr, LA.upper_addr))
    b = O.uniform(3, LA.n)
    for name, L in (("A", LA), ("B", LB), ("A again", LA)):
        psi = np.zeros(L.n)
        p = foam_solve("cuFoamCG", L, b, psi, tolerance=1e-10, max_iter=5000, reuse_addressing=0,
                       reduction="reference")
        want = O.plugin_solve(O.CG, L, b, np.zeros(L.n), 1e-10, 5000)
        assert p["nIterations"] == want.n_iterations, name
        assert psi.tobytes() == want.psi.tobytes(), name
    # two meshes in turn, each kept in its own memory: after the first solve
    # of each, no further device matrix is built
    LC = O.grid_lognormal(9, 8, 7, 4)
    bc = O.uniform(2, LC.n)
    foam_solve("cuFoamCG", LA, b, np.zeros(LA.n), tolerance=1e-8, max_iter=5000, reuse_addressing=1)
    foam_solve("cuFoamCG", LC, bc, np.zeros(LC.n), tolerance=1e-8, max_iter=5000, reuse_addressing=2)
    before = matrix_builds()
    for _ in range(3):
        pa = foam_solve("cuFoamCG", LA, b, np.zeros(LA.n), tolerance=1e-8, max_iter=5000, reuse_addressing=1)
        pc = foam_solve("cuFoamCG", LC, bc, np.zeros(LC.n), tolerance=1e-8, max_iter=5000, reuse_addressing=2)
        assert pa["converged"] and pc["converged"]
    assert matrix_builds() == before
