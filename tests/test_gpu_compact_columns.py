"""SELL-32 with compact columns: one-byte codes (CF_FORMAT_SELL_C8) and
16-bit deltas (CF_FORMAT_SELL_D16).

Both change only how the SELL-32 copy stores its columns: a slot's column is
its row plus an entry of a table of the pattern's distinct offsets col - row
(codes), or plus a signed 16-bit delta.  Every fast-order kernel must
therefore produce the same bits as with 32-bit columns -- iteration counts,
residual histories, psi -- in FP64 and in the mixed-precision FP32 sweeps,
for A and A^T, on the 7-point grids, on meshes whose offsets fill most of the
code table, and on random patterns."""
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
    for f in ("sell", "sell8", "sell16"):
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
    assert out["sell"] == out["sell8"] == out["sell16"]
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
    assert out["sell"] == out["sell8"] == out["sell16"]
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
        for f in ("sell", "sell8", "sell16"):
            M.set_format(f)
            ys[f] = (M.spmv(x, row_order="fast").tobytes(), M.spmv(x, transpose=True, row_order="fast").tobytes(),
                     _solve(M, "CG", b, {"reduction": "fast"}))
        assert ys["sell"] == ys["sell8"] == ys["sell16"]
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
        M.set_format("csr")
        y = M.spmv(x, row_order="fast")
        for f in ("sell", "sell16"):   # rows of 33 entries: summed by the whole warp
            M.set_format(f)
            assert M.format()[0] == f
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
    for f in ("csr", "sell", "sell8", "sell16"):
        M.set_format(f)
        assert M.format()[0] == f
        out[f] = (M.spmv(x, row_order="fast").tobytes(), M.spmv(x, transpose=True, row_order="fast").tobytes())
        if f != "csr":
            out[f] += (_solve(M, "MR", b, {"reduction": "fast", "tolerance": 1e-9}, maxit=5000),)
    assert out["csr"][:2] == out["sell"][:2] == out["sell8"][:2] == out["sell16"][:2]
    assert out["sell"][2] == out["sell8"][2] == out["sell16"][2]
    ref = O.ref_spmv(A, x)
    y = np.frombuffer(out["sell8"][0], dtype=np.float64)
    assert np.allclose(y, ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())


@pytest.mark.parametrize("seed", range(6))
def test_delta16_many_offsets_same_bits(ctx, seed):
    """Patterns with more offsets than the codes' table but every |col - row|
    within 16 bits take the deltas under AUTO (a mesh renumbered inside
    windows of 64 rows: hundreds of offsets; a randomly permuted one): the
    products and fast-order and mixed solves are bit-identical to 32-bit
    columns."""
    base = O.grid_lognormal(24, 20, 16 + seed, 6 + seed)
    rng = np.random.default_rng(seed)
    perm = np.arange(base.n)
    w = 64 if seed % 2 == 0 else base.n
    for s0 in range(0, base.n, w):
        perm[s0:s0 + w] = rng.permutation(perm[s0:s0 + w])
    L = O.permute_ldu(base, perm.astype(np.int32))
    A = O.ldu2csr(L)
    offs = A.cols - np.repeat(np.arange(L.n), np.diff(A.row_offsets))
    assert len(np.unique(offs)) > 32 and np.abs(offs).max() <= 32767
    M = cf.LduMatrix.from_ldu(L, ctx)
    fmt, stored = M.format()
    assert fmt == ("sell16" if stored <= 1.2 * len(A.cols) + 256 else "csr")
    x = O.uniform(7 + seed, L.n)
    b = O.uniform(3 + seed, L.n)
    out = {}
    for f in ("sell", "sell16"):
        M.set_format(f)
        assert M.format()[0] == f
        out[f] = (M.spmv(x, row_order="fast").tobytes(), M.spmv(x, transpose=True, row_order="fast").tobytes(),
                  _solve(M, "CG", b, {"reduction": "fast"}),
                  _solve(M, "MR", b, {"precision": "mixed", "tolerance": 1e-10}))
    assert out["sell"] == out["sell16"]
    assert out["sell"][3][1] == 0


def test_delta16_range_limit(ctx):
    """Offsets beyond 16 bits (a chain of 40,000 cells, cell i < 6,900 also
    coupled to i + 33,000 + i mod 40: 83 distinct offsets up to 33,039): no
    codes and no deltas under AUTO, and asking for the deltas fails."""
    n = 40000
    far = np.arange(6900)
    la = np.concatenate([np.arange(n - 1), far]).astype(np.int32)
    ua = np.concatenate([np.arange(1, n), far + 33000 + far % 40]).astype(np.int32)
    order = np.lexsort((ua, la))
    la, ua = la[order], ua[order]
    w = np.full(len(la), 1.0)
    diag = np.full(n, 4.0)
    L = O.LDU(n, diag, -w, -w, la, ua)
    M = cf.LduMatrix.from_ldu(L, ctx)
    assert M.format()[0] == "sell"
    M.set_format("sell16")
    with pytest.raises(cf.CufoamError, match="16-bit column deltas"):
        M.format()
    M.set_format("auto")
    assert M.format()[0] == "sell"
