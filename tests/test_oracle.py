"""CPU tests of the oracle: pinned to the reference's own ldu2csr (golden
fixtures made by the reference code compiled from source), generator bytes
pinned across hosts, solvers cross-checked against dense direct solves."""
import hashlib
import json
import math
import os

from fractions import Fraction

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN


def test_oracle_ldu2csr_matches_reference_golden(ldu2csr_cases):
    assert len(ldu2csr_cases) >= 8
    for name, (L, ref) in ldu2csr_cases.items():
        A = O.ldu2csr(L)
        assert np.array_equal(A.row_offsets, ref.row_offsets), name
        assert np.array_equal(A.cols, ref.cols), name
        assert A.vals.tobytes() == ref.vals.tobytes(), name


def test_oracle_addressing_matches_golden(ldu2csr_cases):
    for name, (L, _) in ldu2csr_cases.items():
        fresh = O.ldu_addressing(L.n, L.lower_addr, L.upper_addr)
        for a, b in zip(fresh, L._addr):
            assert np.array_equal(a, b), name
        numpy_side = O.LDU(L.n, L.diag, L.lower, L.upper, L.lower_addr, L.upper_addr).addressing()
        for a, b in zip(numpy_side, L._addr):
            assert np.array_equal(a, b), name


def test_reference_ldu2csr_rebuilt_here_agrees(ldu2csr_cases):
    if not O.ref_ldu2csr_available():
        pytest.skip("reference sources not mounted")
    for name, (L, ref) in ldu2csr_cases.items():
        R = O.ref_ldu2csr(L)
        assert np.array_equal(R.row_offsets, ref.row_offsets), name
        assert R.vals.tobytes() == ref.vals.tobytes(), name


def test_generator_bytes_pinned():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_golden", os.path.join(GOLDEN, "gen_golden.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    want = json.load(open(os.path.join(GOLDEN, "generator_checksums.json")))
    got = {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()
           for k, v in gen.generator_inputs().items()}
    assert got == want


def test_addressing_semantics():
    # losort is a stable sort of faces by neighbour; starts are lower bounds
    L = O.grid_const(5, 4, 3)
    ls, lst, ost = L.addressing()
    nbr = L.upper_addr[ls]
    assert np.all(np.diff(nbr) >= 0)
    for c in range(L.n):
        seg = ls[lst[c]:lst[c + 1]]
        assert np.all(L.upper_addr[seg] == c)
        assert np.all(np.diff(seg) > 0)
        assert np.all(L.lower_addr[ost[c]:ost[c + 1]] == c)
    with pytest.raises(ValueError):
        O.ldu_addressing(3, np.array([1, 0], np.int32), np.array([2, 2], np.int32))
    with pytest.raises(ValueError):
        O.ldu_addressing(3, np.array([1], np.int32), np.array([1], np.int32))


def test_grid_sizes_match_configs():
    assert O.grid_addressing(64, 64, 1)[0].shape[0] == 8064
    assert O.n_faces(128, 128, 128) == 6_242_304
    assert O.n_faces(256, 256, 256) == 50_135_040
    assert O.n_faces(96, 96, 96) == 2_626_560


def test_elementary_functions():
    from cufoam_gb300 import workloads as W
    L = W.lib()
    for x in np.linspace(-30, 30, 301):
        assert abs(L.wl_exp(x) / math.exp(x) - 1) < 5e-15
        assert abs(L.wl_sin(x) - math.sin(x)) < 5e-15
        assert abs(L.wl_cos(x) - math.cos(x)) < 5e-15
    for x in np.geomspace(1e-300, 1e300, 301):
        assert abs(L.wl_log(x) - math.log(x)) <= 5e-15 * max(1.0, abs(math.log(x)))


def test_numpy_addressing_matches_oracle_restatement():
    for L in (O.grid_const(7, 5, 3), O.grid_convdiff(6, 5, 4, 2)[0],
              O.permute_ldu(O.grid_lognormal(5, 4, 3, 1), O.permutation(2, 60))):
        mine = L.addressing()
        ref = O.ldu_addressing(L.n, L.lower_addr, L.upper_addr)
        for a, b in zip(mine, ref):
            assert np.array_equal(a, b)


def test_lognormal_and_convdiff_properties():
    L = O.grid_lognormal(6, 5, 4, 3)
    A = O.ldu2csr(L).dense()
    assert np.allclose(A, A.T)
    assert np.all(np.linalg.eigvalsh(A) > 0)
    # diagonal = |off-diagonal| row sum (+ positive wall terms on wall cells)
    off = np.abs(A - np.diag(np.diag(A))).sum(1)
    assert np.all(np.diag(A) >= off * (1 - 1e-14))
    n_off = (np.abs(A) > 0).sum(1) - 1
    assert np.all(np.diag(A)[n_off < 6] > off[n_off < 6])
    cd, stats = O.grid_convdiff(6, 5, 4, 4, pe_max=10.0)
    B = O.ldu2csr(cd).dense()
    assert not np.allclose(B, B.T)
    assert abs(stats["pe_max"] - 10.0) < 1e-12
    # M-matrix: positive diagonal, non-positive off-diagonals, weak row dominance
    assert np.all(np.diag(B) > 0)
    assert np.all(B - np.diag(np.diag(B)) <= 0)
    assert np.all(np.diag(B) - np.abs(B - np.diag(np.diag(B))).sum(1) > -1e-9)


def test_permute_ldu_is_similarity():
    L = O.grid_lognormal(4, 3, 3, 5)
    perm = O.permutation(3, L.n)
    P = O.permute_ldu(L, perm)
    A = O.ldu2csr(L).dense()
    B = O.ldu2csr(P).dense()
    Pm = np.zeros((L.n, L.n))
    Pm[perm, np.arange(L.n)] = 1.0
    assert np.allclose(Pm @ A @ Pm.T, B)


def test_norm_factor_zero_psi_is_source_norm():
    L = O.grid_const(16, 16, 1)
    A = O.ldu2csr(L)
    b = O.uniform(1, L.n)
    nf = O.norm_factor(A, b, np.zeros(L.n))
    assert nf == O.ref_dot(b, b) ** 0.5 + 1e-20


def fma(a, b, c):
    """Correctly rounded a*b + c (exact rational arithmetic)."""
    return float(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def test_ref_spmv_row_order():
    # rows longer than 8 exercise the 8-lane FMA accumulation
    L = O.grid_const(3, 3, 1)
    A = O.ldu2csr(L)
    x = O.uniform(3, L.n)
    assert np.allclose(O.ref_spmv(A, x), A.dense() @ x, rtol=1e-14, atol=1e-14)
    rng = np.random.default_rng(0)
    n = 12
    ro = np.arange(0, n * n + 1, n, dtype=np.int32)
    cols = np.tile(np.arange(n, dtype=np.int32), n)
    vals = rng.standard_normal(n * n)
    D = O.CSR(ro, cols, vals)
    x = rng.standard_normal(n)
    y = O.ref_spmv(D, x)
    row = vals[:n]
    t = [0.0] * 8
    for l in range(8):
        acc = 0.0
        for j in range(l, n, 8):
            acc = fma(row[j], x[j], acc)
        t[l] = acc
    want = ((t[0] + t[4]) + (t[2] + t[6])) + ((t[1] + t[5]) + (t[3] + t[7]))
    assert y[0] == want


@pytest.mark.parametrize("name", list(O.SOLVER_NAMES))
def test_oracle_solvers_converge_to_direct_solution(name):
    kind = O.SOLVER_NAMES[name]
    L = O.grid_lognormal(8, 7, 1, 21) if kind != O.BICG else O.grid_convdiff(8, 7, 1, 22)[0]
    A = O.ldu2csr(L)
    b = O.uniform(2, L.n)
    x0 = np.zeros(L.n)
    r = O.plugin_solve(kind, L, b, x0, 1e-10, 200000)
    xd = np.linalg.solve(A.dense(), b)
    assert r.final_residual <= 1e-10 * (2.0 if kind == O.JMR else 1.0) or r.n_iterations == 200000
    assert np.linalg.norm(r.psi - xd) / np.linalg.norm(xd) < 1e-7
    assert r.history.shape[0] == r.n_iterations + 1
    assert abs(O.true_residual_norm(A, b, r.psi) - np.linalg.norm(b - A.dense() @ r.psi)) < 1e-12


def test_cg_iteration_count_c1():
    L = O.grid_const(64, 64, 1)
    b = O.uniform(1, L.n)
    r = O.plugin_solve(O.CG, L, b, np.zeros(L.n), 1e-6, 10000)
    assert 150 <= r.n_iterations <= 180
    assert r.final_residual <= 1e-6


def test_bicg_breakdown_detected():
    # A = [[0,1],[1,0]]: (p*, A p) = 2 r0 r1 = 0 for r0 = (1, 0) -> xi = inf
    # is not a breakdown (|xi| large); use a tiny rho instead: b = (1e-6, 0)
    L = O.LDU(2, np.array([0.0, 0.0]), np.array([1.0]), np.array([1.0]),
              np.array([0], np.int32), np.array([1], np.int32))
    A = O.ldu2csr(L)
    At = O.ldu2csr(L.transposed())
    b = np.array([1e-6, 1e-6])
    r = O.solve(O.BICG, A, b, np.zeros(2), 1e-30, 10, At=At)
    # xi = (r,r*)/(p*,Ap) = 2e-12 / 2e-12 = 1: no breakdown; then converges
    assert not r.breakdown
    b2 = np.array([1e-6, -1e-6])
    r2 = O.solve(O.BICG, A, b2, np.zeros(2), 1e-30, 10, At=At)
    # (p*, A p) = -2e-12, xi = -1: fine too; a real breakdown needs |xi| < 1e-10
    L3 = O.LDU(2, np.array([1e12, 1e12]), np.array([0.0]), np.array([0.0]),
               np.array([0], np.int32), np.array([1], np.int32))
    A3 = O.ldu2csr(L3)
    r3 = O.solve(O.BICG, A3, np.array([1.0, 1.0]), np.zeros(2), 1e-30, 10, At=O.ldu2csr(L3.transposed()))
    assert r3.breakdown and r3.n_iterations == 0
    assert r2.n_iterations >= 1


def test_richardson_omega_matches_eigen_estimate():
    L = O.grid_lognormal(6, 6, 1, 8)
    A = O.ldu2csr(L)
    b = O.uniform(3, L.n)
    r = O.solve(O.RICHARDSON, A, b, np.zeros(L.n), 1e-8 * np.linalg.norm(b), 100000)
    lmax = np.linalg.eigvalsh(A.dense()).max()
    assert abs(r.lambda_max - lmax) / lmax < 0.05
    assert r.diag_abs_min == np.abs(L.diag).min()
    assert r.omega == 2.0 / (r.lambda_max + r.diag_abs_min)


def test_mrs_equals_mrjacobi_in_exact_arithmetic():
    L = O.grid_lognormal(7, 6, 1, 9)
    b = O.uniform(4, L.n)
    a = O.plugin_solve(O.MRS, L, b, np.zeros(L.n), 1e-8, 50000)
    c = O.plugin_solve(O.MRJACOBI, L, b, np.zeros(L.n), 1e-8, 50000)
    assert a.n_iterations == c.n_iterations
    assert np.array_equal(a.history, c.history)


def _scaled_csr(A, left, right):
    rows = np.repeat(np.arange(A.n), np.diff(A.row_offsets))
    return O.CSR(A.row_offsets.copy(), A.cols.copy(), left[rows] * A.vals * right[A.cols])


def test_mr_on_the_scaled_matrix_is_mrjacobi_and_jmr():
    # The GPU runs MRJacobi (and MRS) as MR on A D^-1 and JMR as MR on
    # D^-1/2 A D^-1/2: the same iterates as the reference's preconditioned
    # loops up to rounding (x = D^-1 x' and x = D^-1/2 x').
    L, _ = O.grid_convdiff(9, 8, 7, 3, 4.0)
    A = O.ldu2csr(L)
    b = O.uniform(6, L.n)
    d = np.asarray(L.diag, np.float64)
    one, dinv, sd = np.ones(L.n), 1.0 / d, np.sqrt(1.0 / d)
    steps = 40
    want = O.solve(O.MRJACOBI, A, b, np.zeros(L.n), 1e-300, steps)
    got = O.solve(O.MR, _scaled_csr(A, one, dinv), b, np.zeros(L.n), 1e-300, steps)
    assert np.allclose(got.history, want.history, rtol=1e-12, atol=0)
    assert np.allclose(dinv * got.x, want.x, rtol=1e-11, atol=1e-14)
    want = O.solve(O.JMR, A, b, np.zeros(L.n), 1e-300, steps)
    got = O.solve(O.MR, _scaled_csr(A, sd, sd), sd * b, np.zeros(L.n), 1e-300, steps)
    assert np.allclose(got.history, want.history, rtol=1e-12, atol=0)
    assert np.allclose(sd * got.x, want.x, rtol=1e-11, atol=1e-14)
    # and Jacobi's step x += D^-1 r, r -= A D^-1 r is one product with A D^-1
    want = O.solve(O.JACOBI, A, b, np.zeros(L.n), 1e-300, steps)
    AD = _scaled_csr(A, one, dinv).dense()
    x, r = np.zeros(L.n), b.copy()
    for _ in range(steps):
        x, r = x + dinv * r, r - AD @ r
    assert np.allclose(x, want.x, rtol=1e-11, atol=1e-14)
    assert np.isclose(np.linalg.norm(r), want.history[-1], rtol=1e-10)


def test_max_iter_cap_and_loop_semantics():
    L = O.grid_const(16, 16, 1)
    b = O.uniform(1, L.n)
    for kind in (O.CG, O.MR, O.JACOBI, O.RICHARDSON, O.BICG):
        r = O.plugin_solve(kind, L, b, np.zeros(L.n), 1e-14, 7)
        assert r.n_iterations == 7 and r.history.shape[0] == 8
    # already converged: no step, except BiCG which always takes one
    x = np.linalg.solve(O.ldu2csr(L).dense(), b)
    for kind in (O.CG, O.MR, O.JACOBI):
        r = O.plugin_solve(kind, L, b, x, 1e-3, 7)
        assert r.n_iterations == 0
    r = O.plugin_solve(O.BICG, L, b, x, 1e-3, 7)
    assert r.n_iterations == 1


def test_fp32_bicg_diverges_on_upwind_convection_diffusion():
    """Why mixed-precision BiCG does not use FP32 BiCG sweeps: BiCG's
    residual grows transiently on this non-normal system before it
    converges; in FP64 it recovers, with FP32 vectors and accumulation it
    stalls far above the FP64 level (numpy, 48^3, cell Peclet 10; at 64^3
    and above FP32 BiCG diverges outright)."""
    import scipy.sparse as sp
    L, _ = O.grid_convdiff(48, 48, 48, 7, 10.0)
    A = O.ldu2csr(L)
    M = sp.csr_matrix((A.vals, A.cols, A.row_offsets), shape=(L.n, L.n))
    b = O.uniform(8, L.n)

    def bicg(dt, iters):
        Ms, Mt = M.astype(dt), M.T.tocsr().astype(dt)
        x = np.zeros(L.n, dt)
        r = b.astype(dt)
        rs, p, ps = r.copy(), r.copy(), r.copy()
        rho = np.dot(r, rs)
        for _ in range(iters):
            q, qs = Ms @ p, Mt @ ps
            xi = rho / np.dot(ps, q)
            x += xi * p
            r -= xi * q
            rs -= xi * qs
            rho, rho1 = np.dot(r, rs), rho
            p = r + (rho / rho1) * p
            ps = rs + (rho / rho1) * ps
        return np.linalg.norm(b - M @ x.astype(np.float64)) / np.linalg.norm(b)

    assert bicg(np.float64, 800) < 1e-8
    assert bicg(np.float32, 800) > 1e-5


def test_fp32_bicgstab_reaches_inner_tolerance_where_fp32_bicg_fails():
    """The FP32 inner solver of mixed BiCG is BiCGStab: on the same system
    (48^3, cell Peclet 10) FP32 BiCGStab reaches a 1e-4 relative residual,
    which one FP64 refinement sweep then needs, while FP32 BiCG (previous
    test) stalls above 1e-5."""
    import scipy.sparse as sp
    L, _ = O.grid_convdiff(48, 48, 48, 7, 10.0)
    A = O.ldu2csr(L)
    M = sp.csr_matrix((A.vals, A.cols, A.row_offsets), shape=(L.n, L.n))
    b = O.uniform(8, L.n)
    Ms = M.astype(np.float32)
    r = b.astype(np.float32) / np.float32(np.linalg.norm(b))
    rh = r.copy()
    x = np.zeros(L.n, np.float32)
    p = r.copy()
    v = np.zeros(L.n, np.float32)
    rho, alpha, w = np.dot(rh, r), np.float32(1), np.float32(1)
    steps = 0
    for k in range(1, 2000):
        if k > 1:
            p = r + (rho / rho_old) * (alpha / w) * (p - w * v)
        v = Ms @ p
        alpha = rho / np.dot(rh, v)
        s = r - alpha * v
        t = Ms @ s
        w = np.dot(t, s) / np.dot(t, t)
        x += alpha * p + w * s
        r = s - w * t
        rho_old, rho = rho, np.dot(rh, r)
        steps = k
        if np.linalg.norm(r) < 1e-4:
            break
    bn = b / np.linalg.norm(b)
    true_rel = np.linalg.norm(bn - M @ x.astype(np.float64))
    assert steps < 2000 and true_rel < 2e-4


def test_reference_iteration_count_moves_under_one_ulp_source_changes():
    """The reference algorithm's own iteration count on an ill-conditioned
    system moves by more than one step when a single source entry changes by
    one ulp, so no summation order other than the reference's can promise
    +-1 there (the GPU tests hold the fast order to this band).  On the
    constant-coefficient 2-D Poisson system (C1) the count does not move."""
    def counts(kind, L, tol, trials=6):
        b = O.uniform(3, L.n)
        ks = [O.plugin_solve(kind, L, b, np.zeros(L.n), tol, 100000).n_iterations]
        rng = np.random.default_rng(0)
        for _ in range(trials):
            bb = b.copy()
            i = int(rng.integers(L.n))
            bb[i] = np.nextafter(bb[i], np.inf)
            ks.append(O.plugin_solve(kind, L, bb, np.zeros(L.n), tol, 100000).n_iterations)
        return ks
    L = O.grid_lognormal(32, 32, 32, 2)
    cg = counts(O.CG, L, 1e-8)
    mrj = counts(O.MRJACOBI, L, 1e-8)
    assert cg[0] == 356 and max(cg) - min(cg) >= 2, cg
    assert mrj[0] == 277 and max(mrj) - min(mrj) >= 10, mrj
    c1 = counts(O.CG, O.grid_const(64, 64, 1), 1e-6, trials=3)
    assert len(set(c1)) == 1, c1
