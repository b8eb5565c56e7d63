"""Pin of the oracle's solver arithmetic against the reference itself.

The oracle (oracle/oracle.c) restates the reference's solvers with a CPU
emulation of the reference kernels' floating-point order.  Here the same
oracle drivers run a second time on the reference's own device kernels
(gis/SparseSystem/kernels.h, compiled from the reference sources into
oracle/_ref/ref_kernels.cubin and launched through the CUDA driver API by
oracle/refgpu/ref_gpu.c), and every primitive result, residual history,
iteration count and solution must agree bit for bit.  The product's
reference-order kernels are in turn checked bit for bit against the
oracle (tests/test_gpu_core.py), so this closes the chain to the
reference's arithmetic."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refk():
    if not O.reference_kernels.available():
        pytest.skip("the reference's kernels were not compiled (no oracle/_ref/ref_kernels.cubin)")
    with O.reference_kernels(0) as r:
        yield r


def _same(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def _both(refk, fn):
    """fn() on the CPU emulation, then on the reference kernels."""
    O.lib().orc_set_backend(None)
    cpu = fn()
    O.lib().orc_set_backend(refk._g.rg_backend())
    before = refk.launches()
    try:
        gpu = fn()
    finally:
        O.lib().orc_set_backend(None)
    refk.check()
    assert refk.launches() > before, "the reference kernels did not run"
    return cpu, gpu


def _long_rows_csr(n, seed):
    """A random square CSR matrix with 1..24 entries per row (more than the
    reference SpMV's 8 lanes), a nonzero diagonal in every row, columns
    sorted."""
    rng = np.random.default_rng(seed)
    ro = [0]
    cols, vals = [], []
    for i in range(n):
        k = int(rng.integers(0, 24))
        c = np.unique(np.concatenate([rng.integers(0, n, k), [i]]))
        cols.extend(c.tolist())
        v = rng.uniform(-1, 1, c.size)
        v[c == i] = 4.0 + rng.uniform(0, 1)
        vals.extend(v.tolist())
        ro.append(len(cols))
    return O.CSR(np.array(ro, np.int32), np.array(cols, np.int32), np.array(vals, np.float64))


def test_launch_grid_is_the_assumed_one(refk):
    # the oracle's default grid is the reference's LaunchConfig on a GB300
    assert refk.grid == O.GB300_REF_GRID


def test_comparison_detects_a_different_summation_order(refk):
    # a CPU SpMV that sums each row in plain entry order (a planted
    # deviation from the reference's 8-lane tree) must not pass as equal
    A = _long_rows_csr(3000, 5)
    x = O.uniform(21, A.n)
    _, gpu = _both(refk, lambda: O.ref_spmv(A, x))
    plain = np.array([sum(A.vals[j] * x[A.cols[j]] for j in range(A.row_offsets[i], A.row_offsets[i + 1]))
                      for i in range(A.n)])
    assert np.allclose(plain, gpu, rtol=1e-12, atol=1e-12)
    assert not _same(plain, gpu)


@pytest.mark.parametrize("n", [1, 1000, 4096, 400_003])
def test_reductions_match_bitwise(refk, n):
    a = O.uniform(11, n)
    b = O.uniform(12, n)
    for fn in (lambda: O.ref_dot(a, b, refk.grid), lambda: O.ref_sum(a, refk.grid),
               lambda: float(O.lib().orc_ref_distance(a, b, n, refk.grid))):
        cpu, gpu = _both(refk, fn)
        assert _same(cpu, gpu), (n, cpu, gpu)


@pytest.mark.parametrize("case", ["c1", "lognormal", "long_rows"])
def test_spmv_and_residual_match_bitwise(refk, case):
    if case == "c1":
        A = O.ldu2csr(O.grid_const(64, 64))
    elif case == "lognormal":
        A = O.ldu2csr(O.grid_lognormal(24, 20, 16, 2))
    else:
        A = _long_rows_csr(3000, 5)
    x = O.uniform(21, A.n)
    b = O.uniform(22, A.n)
    cpu, gpu = _both(refk, lambda: O.ref_spmv(A, x))
    assert _same(cpu, gpu)
    cpu, gpu = _both(refk, lambda: O.ref_residual(A, b, x))
    assert _same(cpu, gpu)
    cpu, gpu = _both(refk, lambda: O.norm_factor(A, b, x, refk.grid))
    assert _same(cpu, gpu), (cpu, gpu)


def _solve_cases():
    c1 = O.grid_const(64, 64)
    logn = O.grid_lognormal(16, 16, 16, 2)
    conv, _ = O.grid_convdiff(16, 16, 16, 3, 5.0)
    return {"c1": c1, "lognormal16": logn, "convdiff16": conv}


@pytest.mark.parametrize("case", ["c1", "lognormal16"])
@pytest.mark.parametrize("kind", [O.CG, O.JACOBI, O.MR, O.MRJACOBI, O.MRS, O.JMR, O.RICHARDSON])
def test_solvers_match_bitwise(refk, case, kind):
    L = _solve_cases()[case]
    A = O.ldu2csr(L)
    b = O.uniform(3, L.n)
    steps = 150 if kind in (O.CG, O.MR, O.MRJACOBI, O.MRS, O.JMR) else 60
    cpu, gpu = _both(refk, lambda: O.solve(kind, A, b, np.zeros(L.n), 1e-12, steps, refk.grid))
    assert cpu.n_iterations == gpu.n_iterations
    assert _same(cpu.history, gpu.history), (kind, case)
    assert _same(cpu.x, gpu.x), (kind, case)
    if kind == O.RICHARDSON:
        assert _same([cpu.omega, cpu.lambda_max, cpu.diag_abs_min],
                     [gpu.omega, gpu.lambda_max, gpu.diag_abs_min])


def test_bicg_matches_bitwise(refk):
    L = _solve_cases()["convdiff16"]
    A = O.ldu2csr(L)
    At = O.ldu2csr(L.transposed())
    b = O.uniform(3, L.n)
    cpu, gpu = _both(refk, lambda: O.solve(O.BICG, A, b, np.zeros(L.n), 1e-12, 120, refk.grid, At=At))
    assert cpu.n_iterations == gpu.n_iterations and cpu.breakdown == gpu.breakdown
    assert _same(cpu.history, gpu.history)
    assert _same(cpu.x, gpu.x)


def test_plugin_solve_matches_bitwise(refk):
    # the whole cuFoamCG::solve computation: normFactor, CG at tol * normFactor
    L = O.grid_lognormal(20, 20, 20, 7)
    b = O.uniform(8, L.n)
    cpu, gpu = _both(refk, lambda: O.plugin_solve(O.CG, L, b, np.zeros(L.n), 1e-8, 1000, refk.grid))
    assert cpu.n_iterations == gpu.n_iterations
    assert _same([cpu.norm_factor, cpu.initial_residual, cpu.final_residual],
                 [gpu.norm_factor, gpu.initial_residual, gpu.final_residual])
    assert _same(cpu.psi, gpu.psi)


def test_device_resident_reference_cg_matches_the_oracle(refk):
    # the timed device-resident reference CG (the reference's host loop with
    # data kept on the GPU) computes what the oracle's CG computes
    L = O.grid_lognormal(20, 20, 20, 9)
    A = O.ldu2csr(L)
    b = O.uniform(4, L.n)
    O.lib().orc_set_backend(None)
    want = O.solve(O.CG, A, b, np.zeros(L.n), 1e-6, 500, refk.grid)
    x, hist, k, ms = refk.cg_device(A, b, np.zeros(L.n), 1e-6, 500)
    assert k == want.n_iterations and ms > 0
    assert _same(hist, want.history)
    assert _same(x, want.x)
