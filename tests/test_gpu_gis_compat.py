"""libGIS.so stand-in on the GPU, driven the way the cuFoam plugins drive
libGIS (device SparseCSR / Vector containers, gis.h calls), against the
oracle's restatement of the reference drivers: with the reference's
reduction order (CUFOAM_GIS_REDUCTION=reference) the answer, the detail
history and NormFactor are bit-identical; in the fast order
(CUFOAM_GIS_REDUCTION=fast) the iteration count is within the reference's
one-ulp band and the tolerance is met; by default BiCG takes the reference
order."""
import numpy as np
import pytest

import oracle as O
from cufoam_gb300.compat import GisError, GisHarness

pytestmark = pytest.mark.gpu

KIND = {"CG": O.CG, "BiCG": O.BICG, "BiCGAt": O.BICG, "Richardson": O.RICHARDSON, "MR": O.MR,
        "Jacobi": O.JACOBI, "MRJacobi": O.MRJACOBI, "JMR": O.JMR, "MRS": O.MRS}


@pytest.fixture(scope="module")
def gis():
    return GisHarness()


def _system(name):
    L = O.grid_convdiff(12, 10, 8, 3)[0] if name.startswith("BiCG") else O.grid_lognormal(12, 10, 8, 2)
    A = O.ldu2csr(L)
    b = O.uniform(3, L.n)
    return L, A, b


@pytest.fixture
def reference_order(monkeypatch):
    monkeypatch.setenv("CUFOAM_GIS_REDUCTION", "reference")


@pytest.mark.parametrize("name", GisHarness.SOLVERS)
def test_gis_solver_bit_exact_reference_order(gis, ref_grid, reference_order, name):
    L, A, b = _system(name)
    x0 = np.zeros(L.n)
    nf = O.norm_factor(A, b, x0, ref_grid)
    error = 1e-8 * nf
    At = O.ldu2csr(L.transposed()) if name.startswith("BiCG") else None
    want = O.solve(KIND[name], A, b, x0, error, 5000, grid=ref_grid, At=At)
    x, det, flag = gis.solve(name, A.row_offsets, A.cols, A.vals, b, x0, error, 5000,
                             p_real=1e-10 if name.startswith("BiCG") else 0.0)
    assert det.tobytes() == want.history.tobytes()
    assert x.tobytes() == want.x.tobytes()
    assert flag == (want.breakdown if name.startswith("BiCG") else False)


@pytest.fixture
def fast_order(monkeypatch):
    monkeypatch.setenv("CUFOAM_GIS_REDUCTION", "fast")


def _reference_band_abs(kind, A, b, x0, error, max_steps, At, trials=8):
    """(min, max) count of the oracle drivers at the absolute threshold
    `error` on b and on copies with one entry moved by one ulp."""
    ks = [O.solve(kind, A, b, x0, error, max_steps, At=At).n_iterations]
    rng = np.random.default_rng(11)
    for t in range(trials):
        bb = b.copy()
        i = int(rng.integers(len(b)))
        bb[i] = np.nextafter(bb[i], np.inf if t % 2 == 0 else -np.inf)
        ks.append(O.solve(kind, A, bb, x0, error, max_steps, At=At).n_iterations)
    return min(ks), max(ks)


@pytest.mark.parametrize("name", GisHarness.SOLVERS)
def test_gis_solver_fast_order(gis, fast_order, name):
    L, A, b = _system(name)
    x0 = O.uniform(9, L.n, -0.5, 0.5)
    nf = O.norm_factor(A, b, x0)
    error = 1e-8 * nf
    At = O.ldu2csr(L.transposed()) if name.startswith("BiCG") else None
    want = O.solve(KIND[name], A, b, x0, error, 5000, At=At)
    x, det, _ = gis.solve(name, A.row_offsets, A.cols, A.vals, b, x0, error, 5000,
                          p_real=1e-10 if name.startswith("BiCG") else 0.0)
    if not name.startswith("BiCG"):  # BiCG's fast order: convergence only (chaotic paths)
        lo, hi = _reference_band_abs(KIND[name], A, b, x0, error, 5000, At)
        w = hi - lo
        assert lo - 1 - w <= len(det) - 1 <= hi + 1 + w, (len(det) - 1, lo, hi)
    assert det[0] == pytest.approx(want.history[0], rel=1e-13)
    assert det[-1] <= error
    if name == "JMR":   # JMR stops on the D^-1/2-scaled residual
        r = (b - O.ref_spmv(A, x)) / np.sqrt(L.diag)
        assert np.linalg.norm(r) <= 1.5 * error
    else:
        assert O.true_residual_norm(A, b, x) <= 1.5 * error


def test_gis_detail_time_and_limits(gis):
    L, A, b = _system("CG")
    x0 = np.zeros(L.n)
    _, t, _ = gis.solve("CG", A.row_offsets, A.cols, A.vals, b, x0, 1e-30, 25, detail="time")
    assert len(t) == 26 and t[0] == 0.0
    assert np.all(np.diff(t) >= 0) and t[-1] > 0 and t[-1] < 10
    # no detail vector, unlimited steps stopped by the threshold
    x, d, _ = gis.solve("CG", A.row_offsets, A.cols, A.vals, b, x0, 1e-6, 0, detail=None)
    assert len(d) == 0
    assert O.true_residual_norm(A, b, x) <= 1.5e-6


def test_gis_bicg_breakdown_flag(gis):
    L, A, b = _system("BiCG")
    x0 = np.zeros(L.n)
    x, det, flag = gis.solve("BiCG", A.row_offsets, A.cols, A.vals, b, x0, 1e-12, 100, p_real=1e300)
    assert flag is True and len(det) == 1 and np.all(x == 0)


def test_gis_transpose_and_norm_factor(gis, ref_grid, reference_order):
    # LDU-derived: equals the transposed LDU matrix's CSR
    L, A, b = _system("CG")
    shape, ro, co, va = gis.transpose(L.n, L.n, A.row_offsets, A.cols, A.vals)
    T = O.ldu2csr(L.transposed())
    assert shape == (L.n, L.n, A.nnz)
    assert np.array_equal(ro, T.row_offsets) and np.array_equal(co, T.cols)
    assert va.tobytes() == T.vals.tobytes()
    # rectangular, ragged: rows of A^T list A's entries by ascending row
    rng = np.random.default_rng(4)
    nr, nc = 37, 53
    rows = [np.sort(rng.choice(nc, size=rng.integers(0, 9), replace=False)) for _ in range(nr)]
    ro2 = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    co2 = np.concatenate(rows).astype(np.int32)
    va2 = rng.standard_normal(co2.shape[0])
    shape, roT, coT, vaT = gis.transpose(nr, nc, ro2, co2, va2)
    assert shape == (nc, nr, co2.shape[0])
    ent = sorted(((c, i, v) for i in range(nr) for c, v in
                  zip(co2[ro2[i]:ro2[i + 1]], va2[ro2[i]:ro2[i + 1]])), key=lambda e: (e[0], e[1]))
    assert np.array_equal(coT, [e[1] for e in ent])
    assert np.array_equal(vaT, [e[2] for e in ent])
    assert np.array_equal(roT, np.concatenate([[0], np.cumsum(np.bincount(co2, minlength=nc))]))
    # NormFactor in the reference order
    x = O.uniform(2, L.n, 0.0, 3.0)
    assert gis.norm_factor(A.row_offsets, A.cols, A.vals, b, x) == O.norm_factor(A, b, x, ref_grid)


def test_gis_rejects_bad_arguments(gis):
    L, A, b = _system("CG")
    with pytest.raises(GisError) as e:
        gis.solve("CG", A.row_offsets, A.cols, A.vals, b[:-1], np.zeros(L.n - 1), 1e-6, 10)
    assert e.value.code == 2
    bad_cols = A.cols.copy()
    bad_cols[5] = L.n + 7
    with pytest.raises(GisError) as e:
        gis.solve("CG", A.row_offsets, bad_cols, A.vals, b, np.zeros(L.n), 1e-6, 10)
    assert e.value.code == 2
