"""Parity at full size: the 7-point Poisson system at 128^3 (2,097,152 rows,
14,581,760 entries), with constant coefficients (diag 6, off-diagonals -1)
and with seeded lognormal(0,1) face coefficients, solved through the plugin
path (normFactor, tolerance 1e-8 relative to it) by cuFoamCG, cuFoamJacobi
and cuFoamRichardson -- the solvers the reference runs on this system.

* The GPU's reference summation order is the oracle's bits at this size
  too: the whole CG solve (history, psi) against the CPU oracle.
* The default (fast) order against the reference order on the GPU: the
  iteration count within the reference's band under one-ulp source changes
  widened by one step plus its width (a single count, i.e. +-1, for
  constant coefficients), and with equal counts the final relative
  residuals within 1e-12.
* Richardson on the lognormal system diverges in the reference algorithm
  itself (its power-method estimate of the largest eigenvalue, 30 steps, is
  too low there, so omega is too large): both orders stop non-finite at the
  same step, and the fast order reproduces that.
"""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O
from cufoam_gb300 import workloads as W

pytestmark = pytest.mark.gpu

N3 = 128
TOL = 1e-8
MAX_ITER = 400000


@pytest.fixture(scope="module")
def c2(ctx):
    import torch
    out = {}
    for name, make in (("const", lambda: W.grid_const(N3, N3, N3)),
                       ("lognormal", lambda: W.grid_lognormal(N3, N3, N3, 2))):
        L = make()
        out[name] = (L, cf.LduMatrix.from_ldu(L, ctx))
    b = W.uniform(3, N3 ** 3)
    yield out, b, torch.from_numpy(b).cuda()
    for _, M in out.values():
        M.close()


def _solve(M, solver, src, reduction, history=0):
    import torch
    psi = torch.zeros(M.n, dtype=torch.float64, device="cuda")
    perf = cf._TABLE[solver]("p", M, {"tolerance": TOL, "maxIter": MAX_ITER,
                                      "reduction": reduction}).solve(psi, src, history=history)
    torch.cuda.synchronize()
    return perf, psi


def test_c2_reference_order_cg_is_the_oracle(c2, ref_grid):
    systems, b, src = c2
    L, M = systems["const"]
    want = O.plugin_solve(O.CG, L, b, np.zeros(L.n), TOL, MAX_ITER, grid=ref_grid)
    perf, psi = _solve(M, "cuFoamCG", src, "reference", history=1000)
    assert perf.n_iterations == want.n_iterations == 449
    assert perf.history.tobytes() == want.history.tobytes()
    assert psi.cpu().numpy().tobytes() == want.psi.tobytes()
    assert perf.norm_factor == want.norm_factor


def _gpu_band(M, solver, b, ref_k, trials=6):
    """The reference order's counts (the oracle's bits on the GPU) on copies
    of the source with one entry moved by one ulp."""
    import torch
    ks = [ref_k]
    rng = np.random.default_rng(11)
    for t in range(trials):
        bb = b.copy()
        i = int(rng.integers(b.shape[0]))
        bb[i] = np.nextafter(bb[i], np.inf if t % 2 == 0 else -np.inf)
        perf, _ = _solve(M, solver, torch.from_numpy(bb).cuda(), "reference")
        ks.append(perf.n_iterations)
    return min(ks), max(ks)


@pytest.mark.parametrize("case", ["const", "lognormal"])
@pytest.mark.parametrize("solver", ["cuFoamCG", "cuFoamJacobi", "cuFoamRichardson"])
def test_c2_default_order_parity(c2, case, solver):
    import torch
    systems, b, src = c2
    L, M = systems[case]
    ref, x_ref = _solve(M, solver, src, "reference")
    fast, x_fast = _solve(M, solver, src, "auto")       # the plugin's default
    if solver == "cuFoamRichardson" and case == "lognormal":
        # the reference algorithm diverges here; so does the fast order, at
        # the same step
        assert ref.status_name == fast.status_name == "non-finite residual"
        assert fast.n_iterations == ref.n_iterations
        return
    assert ref.converged and fast.converged
    if solver == "cuFoamCG" and case == "lognormal":
        lo, hi = _gpu_band(M, solver, b, ref.n_iterations)
    else:
        lo = hi = ref.n_iterations
    w = hi - lo   # the band widened by its own width (see conftest.assert_fast_order_parity)
    assert lo - 1 - w <= fast.n_iterations <= hi + 1 + w, (fast.n_iterations, ref.n_iterations, lo, hi)
    if fast.n_iterations == ref.n_iterations:
        assert abs(fast.final_residual - ref.final_residual) <= 1e-12
    assert fast.final_residual <= TOL
    rel = float(torch.linalg.norm(x_fast - x_ref) / torch.linalg.norm(x_ref))
    assert rel < 1e-6, rel
    r = src - M.spmv(x_fast, row_order="reference")
    assert float(torch.linalg.norm(r)) / fast.norm_factor <= 1.5 * TOL
