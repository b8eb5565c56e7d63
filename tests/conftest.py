import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAVE_GPU = _have_gpu()


def pytest_collection_modifyitems(config, items):
    if HAVE_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def load_ldu2csr_cases():
    import oracle as O
    z = np.load(os.path.join(GOLDEN, "ldu2csr_cases.npz"))
    out = {}
    for name in z["__names__"]:
        name = str(name)
        g = lambda k: z[f"{name}/{k}"]
        L = O.LDU(int(g("n")[0]), g("diag"), g("lower"), g("upper"), g("lower_addr"),
                  g("upper_addr"))
        L._addr = (g("losort"), g("losort_start"), g("owner_start"))
        ref = O.CSR(g("ref_row_offsets"), g("ref_cols"), g("ref_vals"))
        out[name] = (L, ref)
    return out


@pytest.fixture(scope="session")
def ldu2csr_cases():
    return load_ldu2csr_cases()


@pytest.fixture(scope="session")
def ctx():
    import cufoam_gb300 as cf
    return cf.default_context()


@pytest.fixture(scope="session")
def ref_grid(ctx):
    return ctx.device_info()["reference_grid"]


class Band(tuple):
    """(lo, hi) iteration counts of the reference's one-ulp runs, plus
    `spread`: the largest change of the final relative residual among those
    runs that end at the unperturbed run's count (0 when none does)."""
    spread = 0.0


def reference_band(kind, L, b, x0, tol, max_iter, trials: int = 8, grid=None):
    """(min, max) iteration count of the reference algorithm (the oracle, in
    the reference's summation order) on the given system and on `trials`
    copies whose source has one entry moved by one ulp.  On ill-conditioned
    systems the reference's own count moves by more than one step under such
    a change (CG on a 32^3 lognormal system: 356 -> 357..359; MRJacobi:
    277 -> 254..277), so an implementation with a different summation order
    is held to this band; on well-conditioned systems the band is the single
    reference count and the bar is +-1."""
    import oracle as O
    kw = {} if grid is None else {"grid": grid}
    base = O.plugin_solve(kind, L, b, x0, tol, max_iter, **kw)
    ks = [base.n_iterations]
    spread = 0.0
    rng = np.random.default_rng(11)
    for t in range(trials):
        bb = np.array(b, dtype=np.float64, copy=True)
        i = int(rng.integers(L.n))
        bb[i] = np.nextafter(bb[i], np.inf if t % 2 == 0 else -np.inf)
        r = O.plugin_solve(kind, L, bb, x0, tol, max_iter, **kw)
        ks.append(r.n_iterations)
        if r.n_iterations == base.n_iterations:
            spread = max(spread, abs(r.final_residual - base.final_residual))
    band = Band((min(ks), max(ks)))
    band.spread = spread
    return band


def assert_fast_order_parity(perf, want, band, tol):
    """The fast summation order against the reference order's result `want`
    (iterations, final relative residual): the count within the sampled
    band of the reference's one-ulp counts, widened by one step plus the
    band's own width -- a few samples under-cover the tails (on a skewed
    2,000-entry-row system eight samples gave 119..121, forty gave
    119..124) -- so +-1 exactly where the reference does not move; with the
    same count, the final relative residuals (normalised by normFactor)
    agree within 1e-12, or within twice the change one-ulp source
    perturbations cause in the reference's own final residual where that is
    larger; converged runs meet the tolerance."""
    lo, hi = band
    w = hi - lo
    assert lo - 1 - w <= perf.n_iterations <= hi + 1 + w, (perf.n_iterations, want.n_iterations, tuple(band))
    if perf.n_iterations == want.n_iterations:
        bound = max(1e-12, 2.0 * getattr(band, "spread", 0.0))
        assert abs(perf.final_residual - want.final_residual) <= bound, \
            (perf.final_residual, want.final_residual, bound)
    if want.final_residual <= tol:
        assert perf.final_residual <= tol
