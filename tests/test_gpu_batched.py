"""Batched persistent-cluster CG: every (system, right-hand side) pair must
match an independent FP64 solve of the same system (iteration count within
two, normFactor and initial residual to rounding, true residual at
tolerance)."""
import numpy as np
import pytest

import cufoam_gb300 as cf
import oracle as O
from cufoam_gb300.batch import BatchSolver, c4_systems

pytestmark = pytest.mark.gpu


def _small_batch(n_systems=12, seed=11):
    systems, sizes = c4_systems(n_systems, seed=seed, lo=6, hi=14)
    rhs = [np.stack([O.uniform(100 * s + j, L.n) for j in range(3)]) for s, L in enumerate(systems)]
    return systems, rhs


@pytest.mark.parametrize("config", [(1, 256, 0), (2, 128, 0), (4, 256, 0), (8, 512, 0), (4, 256, 1)])
def test_batched_matches_independent_solves(ctx, config):
    systems, rhs = _small_batch()
    tol, maxit = 1e-8, 5000
    B = BatchSolver(systems, n_rhs=3, context=ctx)
    x, results, ms = B.solve(rhs, tolerance=tol, max_iter=maxit, config=config)
    xs = B.unpack(x)
    for s, L in enumerate(systems):
        A = O.ldu2csr(L)
        for j in range(3):
            res = results[s * 3 + j]
            want = O.plugin_solve(O.CG, L, rhs[s][j], np.zeros(L.n), tol, maxit)
            # a different summation order than the oracle: iteration count
            # within two (CG on system 2, component 2 of this batch takes
            # 82, 83 or 84 steps over 30 random orders of its dot-product
            # sums in plain numpy), both at the tolerance, same normFactor
            # and initial residual to rounding, true residual at the tolerance
            assert abs(res["n_iterations"] - want.n_iterations) <= 2, (s, j)
            assert res["status"] == 0 and res["final_residual"] <= tol
            assert abs(res["norm_factor"] - want.norm_factor) <= 1e-13 * want.norm_factor
            assert abs(res["initial_residual"] - want.initial_residual) <= 1e-13
            true_rel = O.true_residual_norm(A, rhs[s][j], xs[s][j]) / res["norm_factor"]
            assert true_rel <= 1.5 * tol


def test_batched_graph_and_direct_launch_agree(ctx):
    systems, rhs = _small_batch(6, seed=3)
    B = BatchSolver(systems, n_rhs=3, context=ctx)
    x1, r1, _ = B.solve(rhs, tolerance=1e-9, max_iter=3000, use_graph=True)
    x2, r2, _ = B.solve(rhs, tolerance=1e-9, max_iter=3000, use_graph=False)
    assert np.array_equal(x1, x2)
    assert [r["n_iterations"] for r in r1] == [r["n_iterations"] for r in r2]


def test_batched_device_tensors_and_max_iter(ctx):
    import torch
    systems, rhs = _small_batch(5, seed=5)
    B = BatchSolver(systems, n_rhs=3, context=ctx)
    b = torch.from_numpy(B.pack(rhs)).cuda()
    x, res, _ = B.solve(b, tolerance=1e-14, max_iter=7)
    torch.cuda.synchronize()
    assert all(r["n_iterations"] == 7 and r["status"] == 1 for r in res)
    assert x.is_cuda


def test_autotuner_picks_and_caches(ctx, tmp_path, monkeypatch):
    monkeypatch.setenv("CUFOAM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    systems, rhs = _small_batch(8, seed=9)
    B = BatchSolver(systems, n_rhs=3, context=ctx)
    cands = [(1, 256, 0), (4, 256, 0)]
    cfg, entry = B.tune(rhs, tolerance=1e-8, max_iter=2000, candidates=cands)
    assert cfg in cands and len(entry["timings_ms"]) == 2
    B2 = BatchSolver(systems, n_rhs=3, context=ctx)
    cfg2, _ = B2.tune(rhs, tolerance=1e-8, max_iter=2000, candidates=cands)
    assert cfg2 == cfg  # served from the cache


@pytest.mark.parametrize("config", [(1, 256, 0), (4, 256, 0), (8, 128, 0)])
def test_batched_mixed_precision_reaches_fp64_tolerance(ctx, config):
    """FP32 CG sweeps inside FP64 refinement: every (system, rhs) reaches the
    FP64 tolerance on its true residual, and the answer agrees with the FP64
    batched answer to the accuracy the tolerance allows."""
    systems, rhs = _small_batch()
    tol, maxit = 1e-10, 20000
    B = BatchSolver(systems, n_rhs=3, context=ctx)
    x64, r64, _ = B.solve(rhs, tolerance=tol, max_iter=maxit, config=config)
    x32, r32, _ = B.solve(rhs, tolerance=tol, max_iter=maxit, config=config, precision="mixed")
    xs64, xs32 = B.unpack(x64), B.unpack(x32)
    for s, L in enumerate(systems):
        A = O.ldu2csr(L)
        for j in range(3):
            res = r32[s * 3 + j]
            assert res["status"] == 0 and res["final_residual"] <= tol, (s, j, res)
            assert res["norm_factor"] == r64[s * 3 + j]["norm_factor"]
            true_rel = O.true_residual_norm(A, rhs[s][j], xs32[s][j]) / res["norm_factor"]
            assert true_rel <= 1.5 * tol
            err = np.linalg.norm(xs32[s][j] - xs64[s][j]) / np.linalg.norm(xs64[s][j])
            assert err < 1e-6, (s, j, err)


@pytest.mark.parametrize("n_rhs", [1, 2, 4])
@pytest.mark.parametrize("precision", ["FP64", "mixed"])
def test_batched_other_component_counts(ctx, n_rhs, precision):
    """1, 2 and 4 right-hand sides per system (each count has its own row
    layout of the gathered search direction: 8, 16 and 32 bytes per cell):
    every pair reaches the tolerance on its true residual, and FP64 matches
    independent solves in iterations."""
    systems, _ = c4_systems(7, seed=13, lo=6, hi=12)
    rhs = [np.stack([O.uniform(500 + 10 * s + j, L.n) for j in range(n_rhs)])
           for s, L in enumerate(systems)]
    tol, maxit = 1e-9, 20000
    B = BatchSolver(systems, n_rhs=n_rhs, context=ctx)
    x, results, _ = B.solve(rhs, tolerance=tol, max_iter=maxit, precision=precision)
    xs = B.unpack(x)
    for s, L in enumerate(systems):
        A = O.ldu2csr(L)
        for j in range(n_rhs):
            res = results[s * n_rhs + j]
            assert res["status"] == 0 and res["final_residual"] <= tol, (s, j, res)
            true_rel = O.true_residual_norm(A, rhs[s][j], xs[s][j]) / res["norm_factor"]
            assert true_rel <= 1.5 * tol
            if precision == "FP64":
                want = O.plugin_solve(O.CG, L, rhs[s][j], np.zeros(L.n), tol, maxit)
                assert abs(res["n_iterations"] - want.n_iterations) <= 2, (s, j)
