"""GPU parity tests through the C ABI: device ldu2csr against the reference's
own CSR (golden fixtures), SpMV / normFactor / all eight solvers against the
oracle.  In the reference summation order the GPU must reproduce the
oracle's bits exactly; in the fast order the iteration count stays within
the counts the reference algorithm itself takes under one-ulp changes of the
source (widened by one step plus the band's width; a single count, i.e.
+-1, on well-conditioned systems), and with equal counts the final relative
residuals agree within 1e-12 (or the reference's own one-ulp spread)."""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O
from conftest import assert_fast_order_parity, reference_band

pytestmark = pytest.mark.gpu

REL_RES_TOL = 1e-12   # |final relative residual (GPU) - (oracle)|


def _matrix(ctx, L, with_addressing=False):
    return cf.LduMatrix.from_ldu(L, ctx, with_addressing=with_addressing)


# ---------------------------------------------------------------------------
# ldu2csr
# ---------------------------------------------------------------------------
def test_ldu2csr_bit_exact_vs_reference(ctx, ldu2csr_cases):
    for name, (L, ref) in ldu2csr_cases.items():
        for given in (False, True):
            M = _matrix(ctx, L, with_addressing=given)
            ro, cols, vals = M.to_csr()
            assert np.array_equal(ro, ref.row_offsets), (name, given)
            assert np.array_equal(cols, ref.cols), (name, given)
            assert vals.tobytes() == ref.vals.tobytes(), (name, given)
            # A^T on the same pattern == ldu2csr of the swapped LDU
            rot, colt, valt = M.to_csr(transpose=True)
            T = O.ldu2csr(L.transposed())
            assert np.array_equal(rot, T.row_offsets) and np.array_equal(colt, T.cols)
            assert valt.tobytes() == T.vals.tobytes(), name
            M.close()


def test_ldu2csr_from_device_tensors(ctx):
    import torch
    L = O.grid_lognormal(9, 7, 5, 31)
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(L, k))).cuda()
           for k in ("diag", "lower", "upper", "lower_addr", "upper_addr")}
    M = cf.LduMatrix(L.n, dev["diag"], dev["lower"], dev["upper"], dev["lower_addr"],
                     dev["upper_addr"], context=ctx)
    ro, cols, vals = M.to_csr()
    R = O.ldu2csr(L)
    assert np.array_equal(ro, R.row_offsets) and np.array_equal(cols, R.cols)
    assert vals.tobytes() == R.vals.tobytes()


def test_update_values_keeps_pattern(ctx):
    L = O.grid_lognormal(8, 6, 4, 1)
    L2 = O.grid_lognormal(8, 6, 4, 2)
    M = _matrix(ctx, L)
    M.update_values(L2.diag, L2.lower, L2.upper)
    ro, cols, vals = M.to_csr()
    assert vals.tobytes() == O.ldu2csr(L2).vals.tobytes()


def test_bad_addressing_is_rejected(ctx):
    d = np.ones(3)
    v = np.ones(2)
    bad = [
        (np.array([1, 0], np.int32), np.array([2, 2], np.int32)),   # owners not sorted
        (np.array([0, 1], np.int32), np.array([0, 2], np.int32)),   # owner == neighbour
        (np.array([0, 1], np.int32), np.array([1, 3], np.int32)),   # out of range
    ]
    for la, ua in bad:
        with pytest.raises(cf.CufoamError) as e:
            cf.LduMatrix(3, d, v, v, la, ua, context=ctx)
        assert e.value.status == 4
    # losortStart covering one face fewer than n_faces: the entry count would
    # not be n + 2F, which the reference's fixed-size CSR cannot hold
    la, ua = np.array([0, 1], np.int32), np.array([1, 2], np.int32)
    with pytest.raises(cf.CufoamError) as e:
        cf.LduMatrix(3, d, v, v, la, ua, losort=np.array([0, 1], np.int32),
                     losort_start=np.array([0, 0, 1, 1], np.int32),
                     owner_start=np.array([0, 1, 2, 2], np.int32), context=ctx)
    assert e.value.status == 4
    # out-of-range losort entry
    with pytest.raises(cf.CufoamError):
        cf.LduMatrix(3, d, v, v, la, ua, losort=np.array([0, 5], np.int32),
                     losort_start=np.array([0, 0, 1, 2], np.int32),
                     owner_start=np.array([0, 1, 2, 2], np.int32), context=ctx)


# ---------------------------------------------------------------------------
# SpMV and normFactor
# ---------------------------------------------------------------------------
def _star_ldu(n):
    """Cell 0 coupled to every other cell: one row of n entries (longer
    than a warp's staging buffer) plus short rows."""
    la = np.zeros(n - 1, np.int32)
    ua = np.arange(1, n, dtype=np.int32)
    rng = np.random.default_rng(5)
    return O.LDU(n, rng.standard_normal(n) + 10, rng.standard_normal(n - 1),
                 rng.standard_normal(n - 1), la, ua)


def _skewed_ldu(n, seed, hubs=40, spd=True):
    """A chain of n cells plus `hubs` hub cells coupled to 40..2,000 random
    higher-numbered cells (power-law-like degrees): rows from 2 to ~2,000
    entries, so 32-row chunks mix short and long rows.  Symmetric
    coefficients and a dominant diagonal make it SPD."""
    rng = np.random.default_rng(seed)
    edges = {(i, i + 1) for i in range(n - 1)}
    hub_cells = rng.choice(n // 2, size=hubs, replace=False)
    for h in hub_cells:
        deg = int(min(n - h - 1, 40 * (1 + rng.pareto(1.2)), 2000))
        for j in rng.choice(np.arange(h + 1, n), size=deg, replace=False):
            edges.add((int(h), int(j)))
    e = np.array(sorted(edges), dtype=np.int32)
    la, ua = e[:, 0].copy(), e[:, 1].copy()
    w = rng.uniform(0.5, 1.5, size=len(e))
    up = -w
    lo = -w if spd else -w * rng.uniform(0.5, 1.5, size=len(e))
    diag = np.ones(n)
    np.add.at(diag, la, np.abs(up) + np.abs(lo))
    np.add.at(diag, ua, np.abs(up) + np.abs(lo))
    return O.LDU(n, diag, lo, up, la, ua)


SPMV_CASES = {"c1": lambda: O.grid_const(64, 64, 1),
              "lognormal": lambda: O.grid_lognormal(20, 17, 9, 3),
              "convdiff": lambda: O.grid_convdiff(16, 15, 14, 4)[0],
              "star": lambda: _star_ldu(3000),
              "skewed": lambda: _skewed_ldu(20000, 3, spd=False),
              "permuted": lambda: O.permute_ldu(O.grid_lognormal(11, 10, 9, 6), O.permutation(6, 990)),
              }


@pytest.mark.parametrize("case", ["c1", "lognormal", "convdiff", "star", "skewed", "permuted"])
def test_spmv_bit_exact(ctx, case):
    L = SPMV_CASES[case]()
    M = _matrix(ctx, L)
    x = O.uniform(7, L.n)
    A = O.ldu2csr(L)
    assert M.spmv(x).tobytes() == O.ref_spmv(A, x).tobytes()
    T = O.ldu2csr(L.transposed())
    assert M.spmv(x, transpose=True).tobytes() == O.ref_spmv(T, x).tobytes()
    # FMA-chain order: same values to rounding
    y = M.spmv(x, row_order="fast")
    ref = O.ref_spmv(A, x)
    assert np.allclose(y, ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())


@pytest.mark.parametrize("case", ["c1", "lognormal", "convdiff", "star", "skewed", "permuted", "ragged"])
def test_spmv_formats_agree(ctx, case):
    """The fast kernels read CSR (warp-chunk staging) or the SELL-32 copy
    with 32-bit columns or one-byte column codes; all sum each row of up to
    32 entries as one FMA chain in entry order and each longer row with the
    whole warp in the same lane partition, so they agree exactly (zeros up
    to sign), for A and A^T, and after a value update.  AUTO takes the codes
    when the pattern has at most 32 distinct offsets col - row (the grids),
    else 16-bit deltas when the offsets fit (the randomly permuted mesh;
    asking for the codes there fails); the star's and the skewed matrix's
    long rows are summed by the whole warp over 16-bit deltas too."""
    L = SPMV_CASES[case]() if case != "ragged" else O.grid_lognormal(7, 5, 3, 9)  # 105 rows
    M = _matrix(ctx, L)
    fmt, stored = M.format()
    nnz = M.shape()[2]
    A = O.ldu2csr(L)
    offsets = np.unique(A.cols - np.repeat(np.arange(L.n), np.diff(A.row_offsets)))
    coded = len(np.union1d(offsets, [0])) <= 32
    if case in ("star", "skewed"):
        assert fmt == "csr" and stored == nnz      # padding to the long row: too much
    else:   # the permuted mesh's offsets all fit 16 bits
        assert fmt == ("sell8" if coded else "sell16") and nnz <= stored <= 1.2 * nnz + 256
    assert coded == (case not in ("permuted", "star", "skewed"))   # 1,627 / 5,999 / 13,845 offsets
    x = O.uniform(7, L.n)
    ref = O.ref_spmv(A, x)
    ys = {}
    for f in ("csr", "sell", "sell8", "sell16"):
        if f == "sell8" and not coded:
            with pytest.raises(cf.CufoamError, match="32 distinct column offsets"):
                M.set_format(f)
                M.format()
            continue
        M.set_format(f)
        assert M.format()[0] == f
        ys[f] = (M.spmv(x, row_order="fast"), M.spmv(x, transpose=True, row_order="fast"))
    for f in ys:
        assert np.array_equal(ys["csr"][0], ys[f][0])
        assert np.array_equal(ys["csr"][1], ys[f][1])
    M.set_format("auto")
    assert np.allclose(ys["sell"][0], ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())
    # new coefficients reach the SELL copy
    L2 = O.LDU(L.n, L.diag * 1.5, L.lower * 0.5, L.upper * 0.25, L.lower_addr, L.upper_addr)
    M.update_values(L2.diag, L2.lower, L2.upper)
    ref2 = O.ref_spmv(O.ldu2csr(L2), x)
    y2 = M.spmv(x, row_order="fast")
    assert np.allclose(y2, ref2, rtol=1e-14, atol=1e-14 * np.abs(ref2).max())
    M.set_format("csr")
    assert np.array_equal(M.spmv(x, row_order="fast"), y2)


def test_norm_factor(ctx, ref_grid):
    L = O.grid_lognormal(17, 13, 11, 8)
    A = O.ldu2csr(L)
    M = _matrix(ctx, L)
    b = O.uniform(1, L.n)
    for psi in (np.zeros(L.n), O.uniform(2, L.n, 0.0, 3.0)):
        want = O.norm_factor(A, b, psi, ref_grid)
        assert M.norm_factor(b, psi, reduction="reference") == want
        assert abs(M.norm_factor(b, psi) - want) <= 1e-14 * want
    # OpenFOAM's L1 normFactor
    psi = O.uniform(2, L.n, 0.0, 3.0)
    Ad = A.dense() if L.n < 3000 else None
    rs = np.array([A.vals[A.row_offsets[i]:A.row_offsets[i + 1]].sum() for i in range(L.n)])
    xbar = psi.mean()
    want = np.abs(O.ref_spmv(A, psi) - rs * xbar).sum() + np.abs(b - rs * xbar).sum() + 1e-20
    assert abs(M.norm_factor(b, psi, norm_type="openfoam") - want) <= 1e-12 * want
    del Ad


# ---------------------------------------------------------------------------
# solvers
# ---------------------------------------------------------------------------
CASES = {
    "c1": (lambda: O.grid_const(64, 64, 1), 1e-6, 40000),
    "lognormal3d": (lambda: O.grid_lognormal(12, 10, 8, 2), 1e-8, 40000),
}


def _problem(case, kind):
    make, tol, maxit = CASES[case]
    L = make()
    if kind == O.BICG and case == "lognormal3d":
        L = O.grid_convdiff(12, 10, 8, 3)[0]
    b = O.uniform(3, L.n)
    return L, b, tol, maxit


@pytest.mark.parametrize("fmt", ["sell8", "sell", "csr"])
@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("name", list(O.SOLVER_NAMES))
def test_solver_reference_order_is_bit_exact(ctx, ref_grid, name, case, fmt):
    """Reference order: the oracle's bits, whether the rows are read from the
    staged CSR arrays or from the SELL-32 slots."""
    kind = O.SOLVER_NAMES[name]
    L, b, tol, maxit = _problem(case, kind)
    want = O.plugin_solve(kind, L, b, np.zeros(L.n), tol, maxit, grid=ref_grid)
    M = _matrix(ctx, L)
    M.set_format(fmt)
    psi = np.zeros(L.n)
    s = cf.New("p", M, {"solver": "cuFoam" + name, "tolerance": tol, "maxIter": maxit,
                        "reduction": "reference"})
    perf = s.solve(psi, b, history=maxit + 1)
    assert perf.n_iterations == want.n_iterations
    assert perf.norm_factor == want.norm_factor
    assert perf.history.tobytes() == want.history.tobytes()
    assert psi.tobytes() == want.psi.tobytes()
    assert perf.initial_residual == want.initial_residual
    assert perf.final_residual == want.final_residual


@pytest.mark.parametrize("fmt", ["sell8", "sell", "csr"])
@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("name", list(O.SOLVER_NAMES))
def test_solver_fast_order_parity(ctx, name, case, fmt):
    """Fast summation order (FMA-chain rows, tree dot products): the count
    within the reference's one-ulp band, equal final relative residuals
    where the counts agree, the tolerance met on the GPU answer's true
    residual.  BiCG's fast order is opt-in (its default is the reference
    order): its iterates follow the summation order chaotically, so only
    convergence and the true residual are required."""
    kind = O.SOLVER_NAMES[name]
    L, b, tol, maxit = _problem(case, kind)
    want = O.plugin_solve(kind, L, b, np.zeros(L.n), tol, maxit)
    M = _matrix(ctx, L)
    M.set_format(fmt)
    psi = np.zeros(L.n)
    perf = cf._TABLE["cuFoam" + name]("p", M, {"tolerance": tol, "maxIter": maxit,
                                              "reduction": "fast"}).solve(psi, b, history=maxit + 1)
    assert abs(perf.norm_factor - want.norm_factor) <= 1e-14 * want.norm_factor
    h0 = want.history[0]
    early = min(10, len(want.history), len(perf.history))
    assert np.all(np.abs(perf.history[:early] - want.history[:early]) <= REL_RES_TOL * h0)
    if kind == O.BICG:
        assert perf.converged == (want.final_residual <= tol)
    else:
        band = reference_band(kind, L, b, np.zeros(L.n), tol, maxit)
        assert_fast_order_parity(perf, want, band, tol)
    A = O.ldu2csr(L)
    if kind == O.JMR:  # JMR stops on the D^-1/2-scaled residual
        r = b - O.ref_spmv(A, psi)
        true_rel = np.linalg.norm(r / np.sqrt(L.diag)) / perf.norm_factor
    else:
        true_rel = O.true_residual_norm(A, b, psi) / perf.norm_factor
    assert true_rel <= 1.5 * tol


@pytest.mark.parametrize("case", ["convdiff_pe10", "convdiff_pe3"])
def test_bicg_defaults_to_the_reference_order(ctx, ref_grid, case):
    """cuFoamBiCG without a `reduction` entry runs the reference's summation
    order (CF_REDUCE_AUTO): the oracle's bits, including on a
    convection-diffusion system where summation orders take different paths."""
    L = O.grid_convdiff(12, 10, 8, 3)[0] if case == "convdiff_pe10" else O.grid_convdiff(20, 18, 16, 3, 3.0)[0]
    b = O.uniform(3, L.n)
    tol, maxit = 1e-8, 40000
    want = O.plugin_solve(O.BICG, L, b, np.zeros(L.n), tol, maxit, grid=ref_grid)
    M = _matrix(ctx, L)
    psi = np.zeros(L.n)
    perf = cf.New("p", M, {"solver": "cuFoamBiCG", "tolerance": tol, "maxIter": maxit}).solve(
        psi, b, history=maxit + 1)
    assert perf.n_iterations == want.n_iterations
    assert perf.history.tobytes() == want.history.tobytes()
    assert psi.tobytes() == want.psi.tobytes()


@pytest.mark.parametrize("fmt", ["csr", "sell"])
def test_solvers_on_skewed_rows(ctx, ref_grid, fmt):
    """Rows from 2 to ~2,000 entries (hub cells): the reference order is the
    oracle's bits on both storage formats; the fast order (long rows summed
    by the whole warp) stays within the reference's one-ulp band for CG and
    Jacobi."""
    L = _skewed_ldu(6000, 8)
    b = O.uniform(4, L.n)
    tol, maxit = 1e-9, 20000
    M = _matrix(ctx, L)
    M.set_format(fmt)
    for name, kind in (("cuFoamCG", O.CG), ("cuFoamJacobi", O.JACOBI)):
        want = O.plugin_solve(kind, L, b, np.zeros(L.n), tol, maxit, grid=ref_grid)
        psi = np.zeros(L.n)
        perf = cf._TABLE[name]("p", M, {"tolerance": tol, "maxIter": maxit,
                                        "reduction": "reference"}).solve(psi, b, history=maxit + 1)
        assert perf.n_iterations == want.n_iterations
        assert psi.tobytes() == want.psi.tobytes()
        psi = np.zeros(L.n)
        fast = cf._TABLE[name]("p", M, {"tolerance": tol, "maxIter": maxit}).solve(psi, b)
        band = reference_band(kind, L, b, np.zeros(L.n), tol, maxit, grid=ref_grid)
        assert_fast_order_parity(fast, want, band, tol)
        assert O.true_residual_norm(O.ldu2csr(L), b, psi) / fast.norm_factor <= 1.5 * tol


def test_graph_and_host_loop_agree(ctx):
    L = O.grid_lognormal(16, 16, 8, 4)
    b = O.uniform(5, L.n)
    M = _matrix(ctx, L)
    out = []
    for g in (1, 0):
        psi = np.zeros(L.n)
        p = cf.cuFoamCG("p", M, {"tolerance": 1e-9, "maxIter": 5000, "useGraph": g,
                                 "reduction": "reference"}).solve(psi, b, history=5001)
        out.append((psi, p))
    assert out[0][0].tobytes() == out[1][0].tobytes()
    assert out[0][1].history.tobytes() == out[1][1].history.tobytes()


def test_nonzero_initial_guess_and_device_tensors(ctx, ref_grid):
    import torch
    L = O.grid_lognormal(14, 12, 10, 7)
    b = O.uniform(8, L.n)
    x0 = O.uniform(9, L.n, -0.5, 0.5)
    want = O.plugin_solve(O.CG, L, b, x0, 1e-9, 5000, grid=ref_grid)
    M = _matrix(ctx, L)
    psi = torch.from_numpy(x0.copy()).cuda()
    src = torch.from_numpy(b).cuda()
    perf = cf.cuFoamCG("p", M, {"tolerance": 1e-9, "maxIter": 5000,
                                "reduction": "reference"}).solve(psi, src)
    torch.cuda.synchronize()
    assert perf.n_iterations == want.n_iterations
    assert psi.cpu().numpy().tobytes() == want.psi.tobytes()


def test_status_codes(ctx):
    L = O.grid_const(32, 32, 1)
    b = O.uniform(1, L.n)
    M = _matrix(ctx, L)
    p = cf.cuFoamJacobi("p", M, {"tolerance": 1e-12, "maxIter": 25}).solve(np.zeros(L.n), b)
    assert p.n_iterations == 25 and p.status == 1 and not p.converged
    p = cf.cuFoamCG("p", M, {"tolerance": 1e-6, "maxIter": 1000}).solve(np.zeros(L.n), b)
    assert p.status == 0 and p.converged
    bad = b.copy()
    bad[7] = np.nan
    p = cf.cuFoamCG("p", M, {"tolerance": 1e-6, "maxIter": 100}).solve(np.zeros(L.n), bad)
    assert p.status == 3 and p.n_iterations == 0
    # BiCG breakdown: |xi| < 1e-10 on the first step (SolverSingleGPU.h:629-630)
    L3 = O.LDU(2, np.array([1e12, 1e12]), np.array([0.0]), np.array([0.0]),
               np.array([0], np.int32), np.array([1], np.int32))
    M3 = _matrix(ctx, L3)
    psi = np.zeros(2)
    p = cf.cuFoamBiCG("p", M3, {"tolerance": 1e-30, "maxIter": 10}).solve(psi, np.ones(2))
    assert p.status == 2 and p.n_iterations == 0 and np.all(psi == 0)


def test_time_limit_stops_loop(ctx):
    L = O.grid_lognormal(48, 48, 48, 3)
    b = O.uniform(1, L.n)
    M = _matrix(ctx, L)
    for g in (1, 0):
        p = cf.cuFoamJacobi("p", M, {"tolerance": 1e-15, "maxIter": 10_000_000, "useGraph": g,
                                     "timeLimit": 0.05}).solve(np.zeros(L.n), b)
        assert p.status == 6
        assert 0 < p.n_iterations < 10_000_000


def test_repeated_solves_reuse_workspace(ctx):
    L = O.grid_lognormal(10, 9, 8, 1)
    M = _matrix(ctx, L)
    b = O.uniform(2, L.n)
    res = []
    for _ in range(3):
        psi = np.zeros(L.n)
        res.append(cf.cuFoamMR("p", M, {"tolerance": 1e-8, "maxIter": 20000}).solve(psi, b))
        res[-1].psi = psi
    assert all(r.n_iterations == res[0].n_iterations for r in res)
    assert all(r.psi.tobytes() == res[0].psi.tobytes() for r in res)


def test_handles_outlive_their_context():
    """cf_context_destroy releases its matrices' and batches' memory and
    orphans their handles: calls on them fail with CF_BAD_INPUT, and
    destroying them afterwards (as a garbage collector may) is safe."""
    from cufoam_gb300 import _capi
    from cufoam_gb300.batch import BatchSolver
    lib = _capi.load()
    c = cf.Context(0)
    L = O.grid_const(8, 8, 1)
    M = cf.LduMatrix.from_ldu(L, c)
    B = BatchSolver([L, O.grid_const(6, 5, 1)], n_rhs=1, context=c)
    x = O.uniform(7, L.n)
    assert M.spmv(x).shape == (L.n,)
    c.close()
    y = np.empty(L.n)
    assert lib.cf_spmv(M._h, 0, x.ctypes.data, y.ctypes.data, _capi.CF_MEM_HOST, 0) == _capi.CF_BAD_INPUT
    M.close()
    B.close()


def test_spmv_async_into_device_buffer(ctx):
    import torch
    L = O.grid_lognormal(20, 17, 9, 3)
    M = _matrix(ctx, L)
    x = O.uniform(7, L.n)
    xd = torch.from_numpy(x).cuda()
    yd = torch.full_like(xd, float("nan"))
    out = M.spmv(xd, row_order="fast", out=yd)
    torch.cuda.synchronize()
    assert out is yd
    assert np.array_equal(yd.cpu().numpy(), M.spmv(x, row_order="fast"))
    M.spmv(xd, transpose=True, row_order="reference", out=yd)
    torch.cuda.synchronize()
    assert yd.cpu().numpy().tobytes() == O.ref_spmv(O.ldu2csr(L.transposed()), x).tobytes()
    with pytest.raises(ValueError):
        M.spmv(x, out=yd)



@pytest.mark.parametrize("fmt", ["sell8", "sell", "csr"])
@pytest.mark.parametrize("case", ["c1", "lognormal3d", "lognormal_nonzero_x0"])
def test_small_system_cg_single_launch(ctx, case, fmt):
    """CG on a small system without a residual history runs as one
    cluster-persistent launch (a different summation order again): same
    normFactor and initial residual to rounding, iterations within the
    reference's one-ulp band, the answer's true residual at the tolerance."""
    import torch
    L = O.grid_const(64, 64, 1) if case == "c1" else O.grid_lognormal(18, 16, 14, 5)
    tol, maxit = (1e-6, 40000) if case == "c1" else (1e-9, 40000)
    b = O.uniform(3, L.n)
    x0 = np.zeros(L.n) if case != "lognormal_nonzero_x0" else O.uniform(9, L.n)
    want = O.plugin_solve(O.CG, L, b, x0, tol, maxit)
    band = reference_band(O.CG, L, b, x0, tol, maxit)
    M = _matrix(ctx, L)
    M.set_format(fmt)
    for where in ("host", "device"):
        psi = x0.copy() if where == "host" else torch.from_numpy(x0.copy()).cuda()
        src = b if where == "host" else torch.from_numpy(b).cuda()
        perf = cf.cuFoamCG("p", M, {"tolerance": tol, "maxIter": maxit}).solve(psi, src)
        out = psi if where == "host" else psi.cpu().numpy()
        assert_fast_order_parity(perf, want, band, tol)
        assert abs(perf.norm_factor - want.norm_factor) <= 1e-13 * want.norm_factor
        assert abs(perf.initial_residual - want.initial_residual) <= 1e-13 * want.initial_residual
        assert perf.converged and perf.final_residual <= tol
        true_rel = O.true_residual_norm(O.ldu2csr(L), b, out) / perf.norm_factor
        assert true_rel <= 1.5 * tol


SMALL_SOLVERS = ["cuFoamJacobi", "cuFoamRichardson", "cuFoamMR", "cuFoamMRJacobi", "cuFoamMRS", "cuFoamJMR"]
_SMALL_WANT = {}


def _small_case(name, case):
    """(L, tol, maxit, b, oracle result, band), computed once per case; the
    constant-coefficient 64^2 system's counts do not move under one-ulp
    source changes, so two trials bound its band."""
    key = (name, case)
    if key not in _SMALL_WANT:
        if case == "c1":
            L, tol, maxit = O.grid_const(64, 64, 1), 1e-6, 40000
        elif case == "const3d":
            L, tol, maxit = O.grid_const(12, 12, 12), 1e-8, 40000
        else:
            L, tol, maxit = O.grid_convdiff(14, 12, 10, 5, 1.0)[0], 1e-8, 40000
        kind = O.SOLVER_NAMES[name.replace("cuFoam", "")]
        b = O.uniform(3, L.n)
        want = O.plugin_solve(kind, L, b, np.zeros(L.n), tol, maxit)
        band = reference_band(kind, L, b, np.zeros(L.n), tol, maxit, trials=2 if case == "c1" else 8)
        _SMALL_WANT[key] = (L, tol, maxit, b, want, band)
    return _SMALL_WANT[key]


# (solver, system, format): the 64^2 system in SELL-32, the 3-D ones in both
# formats; Richardson is registered for symmetric matrices only
SMALL_CASES = [(name, case, fmt) for name in SMALL_SOLVERS
               for case, fmt in (("c1", "sell"), ("const3d", "sell"), ("const3d", "csr"),
                                 ("convdiff", "sell"), ("convdiff", "csr"))
               if not (case == "convdiff" and name == "cuFoamRichardson")]


@pytest.mark.parametrize("name,case,fmt", SMALL_CASES)
def test_small_system_solvers_single_launch(ctx, name, case, fmt):
    """Jacobi, Richardson and the MR family on a small system without a
    residual history run as one cluster-persistent launch (k_small_solve):
    the same normFactor and initial residual to rounding, iterations within
    the reference's one-ulp band, Richardson's power-method factor to
    rounding, the answer's true residual at the tolerance."""
    import torch
    L, tol, maxit, b, want, band = _small_case(name, case)
    M = _matrix(ctx, L)
    M.set_format(fmt)
    for where in ("host", "device"):
        psi = np.zeros(L.n) if where == "host" else torch.zeros(L.n, dtype=torch.float64, device="cuda")
        src = b if where == "host" else torch.from_numpy(b).cuda()
        perf = cf._TABLE[name]("p", M, {"tolerance": tol, "maxIter": maxit}).solve(psi, src)
        out = psi if where == "host" else psi.cpu().numpy()
        assert_fast_order_parity(perf, want, band, tol)
        assert abs(perf.norm_factor - want.norm_factor) <= 1e-13 * want.norm_factor
        assert abs(perf.initial_residual - want.initial_residual) <= 1e-13 * want.initial_residual
        if name == "cuFoamRichardson":
            assert perf.omega == pytest.approx(want.solve.omega, rel=1e-12)
        assert perf.converged and perf.final_residual <= tol
        if name != "cuFoamJMR":   # JMR's recorded residual is the scaled one
            true_rel = O.true_residual_norm(O.ldu2csr(L), b, out) / perf.norm_factor
            assert true_rel <= 1.5 * tol


@pytest.mark.parametrize("offset", [0, 1])
def test_cg_odd_size_and_unaligned_device_vectors(ctx, offset):
    """The fast CG prep pass takes element pairs as 16-byte loads when psi and
    the work vectors are 16-byte aligned, and a scalar loop otherwise; an odd
    row count leaves one element outside the pairs.  Both paths give the
    same iterates (one FMA per element either way)."""
    import torch
    L = O.grid_lognormal(11, 9, 7, 3)            # 693 rows
    b = O.uniform(5, L.n)
    tol, maxit = 1e-10, 5000
    M = _matrix(ctx, L)
    want = O.plugin_solve(O.CG, L, b, np.zeros(L.n), tol, maxit)
    buf = torch.zeros(L.n + 1, dtype=torch.float64, device="cuda")
    psi = buf[offset:offset + L.n]               # offset 1: 8 bytes past a 16-byte boundary
    src = torch.from_numpy(b).cuda()
    perf = cf.cuFoamCG("p", M, {"tolerance": tol, "maxIter": maxit}).solve(psi, src, history=maxit + 1)
    torch.cuda.synchronize()
    band = reference_band(O.CG, L, b, np.zeros(L.n), tol, maxit)
    assert_fast_order_parity(perf, want, band, tol)
    x = psi.cpu().numpy()
    assert O.true_residual_norm(O.ldu2csr(L), b, x) / perf.norm_factor <= 1.5 * tol
    if offset == 1:   # the same bits as the aligned solve
        buf2 = torch.zeros(L.n, dtype=torch.float64, device="cuda")
        p2 = cf.cuFoamCG("p", M, {"tolerance": tol, "maxIter": maxit}).solve(buf2, src, history=maxit + 1)
        torch.cuda.synchronize()
        assert p2.history.tobytes() == perf.history.tobytes()
        assert buf2.cpu().numpy().tobytes() == x.tobytes()
