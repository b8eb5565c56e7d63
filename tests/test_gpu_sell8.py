"""SELL-32 with one-byte column codes (CF_FORMAT_SELL_C8).

The codes change only how the SELL-32 copy stores its columns: a slot's
column is its row plus an entry of a table of the pattern's distinct offsets
col - row.  Every fast-order kernel must therefore produce the same bits as
with 32-bit columns -- iteration counts, residual histories, psi -- in FP64
and in the mixed-precision FP32 sweeps, for A and A^T, on the 7-point grids
and on a mesh whose offsets fill most of the table."""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O

pytestmark = pytest.mark.gpu


def _solve(M, name, b, opts, transpose=False, maxit=40000):
    psi = np.zeros(M.shape()[0])
    o = {"tolerance": 1e-8, "maxIter": maxit}
    o.update(opts)
    perf = cf._TABLE["cuFoam" + name]("p", M, o).solve(psi, b, history=maxit + 1, transpose=transpose)
    return perf.n_iterations, perf.status, perf.history.tobytes(), psi.tobytes()


def _both(M, name, b, opts, transpose=False):
    out = {}
    for f in ("sell", "sell8"):
        M.set_format(f)
        out[f] = _solve(M, name, b, opts, transpose)
        assert M.format()[0] == f
    M.set_format("auto")
    return out


@pytest.mark.parametrize("name", ["CG", "PCG", "BiCG", "Jacobi", "Richardson", "MR", "MRJacobi", "MRS", "JMR"])
def test_fp64_fast_order_same_bits(ctx, name):
    L = O.grid_lognormal(12, 10, 8, 2) if name not in ("BiCG",) else O.grid_convdiff(12, 10, 8, 3)[0]
    b = O.uniform(3, L.n)
    M = cf.LduMatrix.from_ldu(L, ctx)
    assert M.format()[0] == "sell8"
    out = _both(M, name, b, {"reduction": "fast"})
    assert out["sell"] == out["sell8"]
    assert out["sell"][0] > 5


@pytest.mark.parametrize("name", ["CG", "BiCG", "MR", "MRJacobi", "JMR"])
@pytest.mark.parametrize("transpose", [False, True])
def test_mixed_sweeps_same_bits(ctx, name, transpose):
    if name == "CG" and transpose:
        pytest.skip("CG solves symmetric systems")
    L = O.grid_lognormal(12, 10, 8, 2) if name == "CG" else O.grid_convdiff(14, 12, 10, 9, 4.0)[0]
    b = O.uniform(5, L.n)
    M = cf.LduMatrix.from_ldu(L, ctx)
    out = _both(M, name, b, {"precision": "mixed", "tolerance": 1e-10}, transpose)
    assert out["sell"] == out["sell8"]
    assert out["sell"][1] == 0


def test_many_offsets_and_value_update(ctx):
    """A 12x10x8 mesh whose rows are randomly renumbered inside windows of 3
    rows: 31 distinct offsets, one short of the codes' limit.  The plain
    SpMV and a CG solve agree bit for bit with the 32-bit columns, before
    and after new coefficient values."""
    base = O.grid_lognormal(12, 10, 8, 6)
    rng = np.random.default_rng(11)
    perm = np.arange(base.n)
    for s in range(0, base.n, 3):
        perm[s:s + 3] = rng.permutation(perm[s:s + 3])
    L = O.permute_ldu(base, perm.astype(np.int32))
    A = O.ldu2csr(L)
    offs = np.unique(A.cols - np.repeat(np.arange(L.n), np.diff(A.row_offsets)))
    assert len(offs) == 31
    M = cf.LduMatrix.from_ldu(L, ctx)
    assert M.format()[0] == "sell8"
    x = O.uniform(7, L.n)
    b = O.uniform(3, L.n)
    for step in range(2):
        ys = {}
        for f in ("sell", "sell8"):
            M.set_format(f)
            ys[f] = (M.spmv(x, row_order="fast").tobytes(), M.spmv(x, transpose=True, row_order="fast").tobytes(),
                     _solve(M, "CG", b, {"reduction": "fast"}))
        assert ys["sell"] == ys["sell8"]
        ref = O.ref_spmv(O.ldu2csr(L), x)
        y = np.frombuffer(ys["sell8"][0], dtype=np.float64)
        assert np.allclose(y, ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())
        L = O.LDU(L.n, L.diag * 1.25, L.lower * 0.5, L.upper * 0.5, L.lower_addr, L.upper_addr)
        M.update_values(L.diag, L.lower, L.upper)


def _band_ldu(n, strides):
    """Cell i coupled to i + k for every k in `strides`: offsets 0 and +-k,
    1 + 2 len(strides) of them; diagonally dominant."""
    la = np.concatenate([np.arange(n - k, dtype=np.int32) for k in strides])
    ua = np.concatenate([np.arange(k, n, dtype=np.int32) for k in strides])
    order = np.lexsort((ua, la))
    la, ua = la[order], ua[order]
    rng = np.random.default_rng(9)
    w = rng.uniform(0.5, 1.5, size=len(la))
    diag = np.ones(n)
    np.add.at(diag, la, 2 * w)
    np.add.at(diag, ua, 2 * w)
    return O.LDU(n, diag, -w, -0.8 * w, la, ua)


@pytest.mark.parametrize("n_strides", [15, 16])
def test_codes_limit(ctx, n_strides):
    """31 offsets take the codes; 33 refuse an explicit request for the
    codes and keep 32-bit columns when SELL-32 is asked for (AUTO takes CSR
    there: rows average more than 32 entries)."""
    L = _band_ldu(5000, list(range(1, 8)) + [50 + 13 * j for j in range(n_strides - 7)])
    M = cf.LduMatrix.from_ldu(L, ctx)
    x = O.uniform(7, L.n)
    if n_strides == 15:
        assert M.format()[0] == "sell8"
        y8 = M.spmv(x, row_order="fast", transpose=True)
        M.set_format("sell")
        assert M.spmv(x, row_order="fast", transpose=True).tobytes() == y8.tobytes()
    else:
        assert M.format()[0] == "csr"
        M.set_format("sell8")
        with pytest.raises(cf.CufoamError, match="at most 32 distinct column offsets"):
            M.format()
        M.set_format("sell")
        assert M.format()[0] == "sell"
        M.set_format("csr")
        y = M.spmv(x, row_order="fast")
        M.set_format("sell")
        assert M.spmv(x, row_order="fast").tobytes() == y.tobytes()


def _random_offset_ldu(seed):
    """A random symmetric pattern whose couplings use a random set of 2..15
    strides (offsets 0 and +-k: at most 31), with cells dropped from some
    couplings, on a ragged size: uneven slices and rows of 1..31 entries."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(40, 3000))
    strides = np.sort(rng.choice(np.arange(1, min(n - 1, 400)), size=int(rng.integers(2, 16)), replace=False))
    la, ua = [], []
    for k in strides:
        keep = rng.random(n - k) < rng.uniform(0.3, 1.0)
        cells = np.arange(n - k)[keep]
        la.append(cells)
        ua.append(cells + k)
    la = np.concatenate(la).astype(np.int32)
    ua = np.concatenate(ua).astype(np.int32)
    order = np.lexsort((ua, la))
    la, ua = la[order], ua[order]
    w = rng.uniform(0.5, 1.5, size=len(la))
    diag = np.ones(n)
    np.add.at(diag, la, 2 * w)
    np.add.at(diag, ua, 2 * w)
    return O.LDU(n, diag, -w, -rng.uniform(0.5, 1.0) * w, la, ua)


@pytest.mark.parametrize("seed", range(12))
def test_random_offset_sets_same_bits(ctx, seed):
    """Random patterns within the codes' limit: the product over the codes
    is bit-identical to the 32-bit columns and to CSR, for A and A^T, and a
    fast-order MR solve takes the same steps to the same bits."""
    L = _random_offset_ldu(seed)
    A = O.ldu2csr(L)
    assert len(np.unique(A.cols - np.repeat(np.arange(L.n), np.diff(A.row_offsets)))) <= 32
    M = cf.LduMatrix.from_ldu(L, ctx)
    x = O.uniform(7 + seed, L.n)
    b = O.uniform(3 + seed, L.n)
    out = {}
    for f in ("csr", "sell", "sell8"):
        M.set_format(f)
        assert M.format()[0] == f
        out[f] = (M.spmv(x, row_order="fast").tobytes(), M.spmv(x, transpose=True, row_order="fast").tobytes())
        if f != "csr":
            out[f] += (_solve(M, "MR", b, {"reduction": "fast", "tolerance": 1e-9}, maxit=5000),)
    assert out["csr"][:2] == out["sell"][:2] == out["sell8"][:2]
    assert out["sell"][2] == out["sell8"][2]
    ref = O.ref_spmv(A, x)
    y = np.frombuffer(out["sell8"][0], dtype=np.float64)
    assert np.allclose(y, ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())
