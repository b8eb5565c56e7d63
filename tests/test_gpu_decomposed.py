"""Decomposed CG on the GPU (cf_solve_decomposed): every rank solves its
subdomain on the device, processor-patch values and inner products move
through gloo on the host.  The ranks run as processes sharing one GPU;
their kernels never wait for one another (all waiting is on the host, in
the exchange and all-reduce callbacks).

Parity: the decomposed solve is the undecomposed one with a different
summation order, so it is held to the reference's (the oracle's) result
on the whole mesh exactly as the fast order is: the iteration count within
the reference's own one-ulp band and the final relative residual within
its spread; normFactor, summed over the ranks, equals the whole mesh's
to rounding."""
import json
import os
import socket
import sys

import numpy as np
import pytest

from conftest import assert_fast_order_parity, reference_band

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

pytestmark = pytest.mark.gpu

TOL, MAXIT = 1e-8, 5000


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case(name):
    from cufoam_gb300 import workloads as W
    if name == "const":
        nx, ny, nz = 24, 20, 16
        L = W.grid_const(nx, ny, nz)
        parts, block = 2, 6
    elif name == "lognormal":
        nx, ny, nz = 20, 18, 16
        L = W.grid_lognormal(nx, ny, nz, 9)
        parts, block = 3, 4
    else:  # slabs: four ranks along z, two processor patches per inner rank
        nx, ny, nz = 32, 32, 32
        L = W.grid_lognormal(nx, ny, nz, 4)
        k = np.repeat(np.arange(nz), nx * ny)
        return L, (k * 4) // nz, W.uniform(13, L.n)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cr = (((i // block) + 2 * (j // block) + (k // block)) % parts).transpose(2, 1, 0).reshape(-1)
    return L, cr, W.uniform(13, L.n)


def _rank_main(rank, world, port, out_dir, case, device_arrays):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import cufoam_gb300 as cf
    from cufoam_gb300.decomposed import ProcessorInterfaces, decompose
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        L, cr, b = _case(case)
        sub = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, cr)[rank]
        ctx = cf.Context(0)
        A = cf.LduMatrix(sub.n, sub.diag, sub.lower, sub.upper, sub.lower_addr, sub.upper_addr,
                         context=ctx)
        s = cf.cuFoamCG("p", A, {"tolerance": TOL, "maxIter": MAXIT},
                        interfaces=ProcessorInterfaces.from_subdomain(sub))
        bl = np.ascontiguousarray(b[sub.cells])
        if device_arrays:
            psi_t = torch.zeros(sub.n, dtype=torch.float64, device="cuda:0")
            p = s.solve(psi_t, torch.from_numpy(bl).cuda(), history=MAXIT + 1)
            torch.cuda.synchronize()
            psi = psi_t.cpu().numpy()
        else:
            psi = np.zeros(sub.n)
            p = s.solve(psi, bl, history=MAXIT + 1)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"k": p.n_iterations, "final": p.final_residual, "init": p.initial_residual,
                       "nf": p.norm_factor, "status": p.status, "hist": p.history.tolist(),
                       "cells": sub.cells.tolist(), "x": psi.tolist(),
                       "n_faces": int(sum(len(q.faces) for q in sub.patches))}, f)
        dist.barrier()
        A.close()
        ctx.close()
    finally:
        dist.destroy_process_group()


def _run(tmp_path, case, world, device_arrays=False):
    import torch.multiprocessing as mp
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path), case, device_arrays),
                       nprocs=world, start_method="spawn")
    return [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]


@pytest.mark.parametrize("case,world,device_arrays", [("const", 2, False), ("lognormal", 3, True),
                                                      ("slabs", 4, False)])
def test_decomposed_cg_matches_the_whole_mesh_reference(tmp_path, case, world, device_arrays):
    import oracle as O
    got = _run(tmp_path, case, world, device_arrays)
    assert all(g["n_faces"] > 0 for g in got)
    for g in got[1:]:     # one solve: all ranks agree bit for bit
        for key in ("k", "final", "init", "nf", "status", "hist"):
            assert g[key] == got[0][key], key
    L, _, b = _case(case)
    want = O.plugin_solve(O.CG, L, b, np.zeros(L.n), TOL, MAXIT)
    g = got[0]
    assert g["nf"] == pytest.approx(want.norm_factor, rel=1e-12)
    assert g["init"] == pytest.approx(want.initial_residual, rel=1e-12)

    class P:
        n_iterations = g["k"]
        final_residual = g["final"]
    band = reference_band(O.CG, L, b, np.zeros(L.n), TOL, MAXIT)
    assert_fast_order_parity(P, want, band, TOL)
    x = np.zeros(L.n)
    for r in got:
        x[np.array(r["cells"])] = r["x"]
    assert g["status"] == 0
    # the assembled solution is the whole mesh's
    A = O.ldu2csr(L)
    assert O.true_residual_norm(A, b, x) <= TOL * want.norm_factor * 1.0001
    assert np.linalg.norm(x - want.psi) <= 1e-6 * np.linalg.norm(want.psi)


def test_decomposed_solve_reports_callback_failures_and_refuses_mixed():
    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    from cufoam_gb300.decomposed import ProcessorComm, ProcessorInterfaces, decompose
    L = W.grid_const(8, 8, 4)
    sub = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper,
                    (np.arange(L.n) >= L.n // 2).astype(int))[0]

    class Failing(ProcessorComm):
        def __init__(self, patches):
            self.slices, self.error, self.group = [], None, None
            self.n_faces = sum(len(p.face_cells) for p in patches)

        def exchange(self, send, recv):
            raise ConnectionError("peer gone")

        def allreduce_sum(self, values):
            pass
    fc, co = sub.interface_arrays()
    ifc = ProcessorInterfaces(fc, co, Failing(sub.patches))
    A = cf.LduMatrix(sub.n, sub.diag, sub.lower, sub.upper, sub.lower_addr, sub.upper_addr)
    for cls in (cf.cuFoamCG, cf.cuFoamBiCG, cf.cuFoamRichardson):
        with pytest.raises(ConnectionError):
            cls("p", A, {"tolerance": 1e-8}, interfaces=ifc).solve(np.zeros(sub.n), np.ones(sub.n))
    with pytest.raises(cf.CufoamError) as e:
        cf.cuFoamCG("p", A, {"tolerance": 1e-8, "precision": "mixed"},
                    interfaces=ifc).solve(np.zeros(sub.n), np.ones(sub.n))
    assert e.value.status == 8     # CF_UNSUPPORTED
    A.close()


# ---------------------------------------------------------------------------
# every solver, three ranks, against the whole mesh
# ---------------------------------------------------------------------------
SOLVERS = [  # (plugin, case, tolerance, maxIter)
    ("cuFoamCG", "sym", 1e-8, 5000),
    ("cuFoamPCG", "sym", 1e-8, 5000),
    ("cuFoamBiCG", "convdiff", 1e-8, 5000),
    ("cuFoamJacobi", "const", 1e-6, 20000),
    ("cuFoamMR", "const", 1e-6, 20000),
    ("cuFoamMRJacobi", "convdiff", 1e-8, 20000),
    ("cuFoamMRS", "convdiff", 1e-8, 20000),
    ("cuFoamJMR", "sym", 1e-6, 20000),
    ("cuFoamRichardson", "const", 1e-6, 20000),
]


def _solver_case(name):
    from cufoam_gb300 import workloads as W
    nx, ny, nz = 14, 12, 10
    if name == "sym":
        L = W.grid_lognormal(nx, ny, nz, 21)
    elif name == "const":
        L = W.grid_const(nx, ny, nz)
    else:
        L, _ = W.grid_convdiff(nx, ny, nz, 5, 1.0)
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cr = (((i // 3) + 2 * (j // 3) + (k // 3)) % 3).transpose(2, 1, 0).reshape(-1)
    return L, cr, W.uniform(17, L.n)


def _solvers_rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import cufoam_gb300 as cf
    from cufoam_gb300.decomposed import ProcessorInterfaces, decompose
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ctx = cf.Context(0)
        res = {}
        for name, case, tol, maxit in SOLVERS:
            L, cr, b = _solver_case(case)
            sub = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, cr)[rank]
            A = cf.LduMatrix(sub.n, sub.diag, sub.lower, sub.upper, sub.lower_addr, sub.upper_addr,
                             context=ctx)
            psi = np.zeros(sub.n)
            p = cf._TABLE[name]("p", A, {"tolerance": tol, "maxIter": maxit},
                                interfaces=ProcessorInterfaces.from_subdomain(sub)).solve(psi, b[sub.cells])
            res[name] = {"k": p.n_iterations, "final": p.final_residual, "init": p.initial_residual,
                         "nf": p.norm_factor, "status": p.status, "omega": p.omega,
                         "cells": sub.cells.tolist(), "x": psi.tolist()}
            A.close()
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump(res, f)
        dist.barrier()
        ctx.close()
    finally:
        dist.destroy_process_group()


@pytest.fixture(scope="module")
def solver_runs(tmp_path_factory):
    import torch.multiprocessing as mp
    d = tmp_path_factory.mktemp("dd_solvers")
    mp.start_processes(_solvers_rank_main, args=(3, _free_port(), str(d)), nprocs=3, start_method="spawn")
    return [json.load(open(d / f"rank{r}.json")) for r in range(3)]


@pytest.mark.parametrize("name,case,tol,maxit", SOLVERS)
def test_every_solver_decomposed_matches_the_whole_mesh(solver_runs, name, case, tol, maxit):
    import cufoam_gb300 as cf
    import oracle as O
    got = [r[name] for r in solver_runs]
    for g in got[1:]:
        for key in ("k", "final", "init", "nf", "status", "omega"):
            assert g[key] == got[0][key], key
    g = got[0]
    L, _, b = _solver_case(case)
    x = np.zeros(L.n)
    for r in got:
        x[np.array(r["cells"])] = r["x"]
    if name == "cuFoamPCG":
        # no reference counterpart: the undecomposed solve of this library
        M = cf.LduMatrix.from_ldu(L)
        psi = np.zeros(L.n)
        want = cf.cuFoamPCG("p", M, {"tolerance": tol, "maxIter": maxit}).solve(psi, b)
        M.close()
        assert abs(g["k"] - want.n_iterations) <= 1
        assert g["nf"] == pytest.approx(want.norm_factor, rel=1e-12)
        assert g["status"] == 0 and g["final"] <= tol
        assert np.linalg.norm(x - psi) <= 1e-5 * np.linalg.norm(psi)
        return
    kind = O.SOLVER_NAMES[name.replace("cuFoam", "")]
    want = O.plugin_solve(kind, L, b, np.zeros(L.n), tol, maxit)
    assert g["nf"] == pytest.approx(want.norm_factor, rel=1e-12)
    assert g["init"] == pytest.approx(want.initial_residual, rel=1e-12)
    if name == "cuFoamRichardson":
        assert g["omega"] == pytest.approx(want.solve.omega, rel=1e-12)

    class P:
        n_iterations = g["k"]
        final_residual = g["final"]
    band = reference_band(kind, L, b, np.zeros(L.n), tol, maxit)
    assert_fast_order_parity(P, want, band, tol)
    assert g["status"] == 0
    assert np.linalg.norm(x - want.psi) <= 1e-5 * np.linalg.norm(want.psi)


# ---------------------------------------------------------------------------
# through the OpenFOAM plugin: a parallel run of the stand-in, processor
# patches as OpenFOAM's processor interfaces, transfers by its Pstream
# ---------------------------------------------------------------------------
def _plugin_rank_main(rank, world, port, out_dir, case):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from cufoam_gb300.decomposed import decompose
    from cufoam_gb300.plugin import ParallelRun, foam_solve_decomposed
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out = {}
        with ParallelRun() as run:
            for name, c in (("cuFoamCG", case), ("cuFoamBiCG", "convdiff"), ("cuFoamRichardson", "const")):
                if c == case:
                    L, cr, b = _case(case)
                else:
                    L, cr, b = _solver_case(c)
                sub = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, cr)[rank]
                psi = np.zeros(sub.n)
                tol = TOL if name != "cuFoamRichardson" else 1e-6
                p = foam_solve_decomposed(name, sub, b[sub.cells], psi, tolerance=tol, max_iter=20000,
                                          symmetric=name != "cuFoamBiCG")
                out[name] = {"k": p["nIterations"], "final": p["finalResidual"], "init": p["initialResidual"],
                             "conv": p["converged"], "cells": sub.cells.tolist(), "x": psi.tolist(),
                             "tol": tol}
            err = None
            try:   # mixed precision has no decomposed form: a FatalError on every rank
                foam_solve_decomposed("cuFoamCG", sub, b[sub.cells], np.zeros(sub.n), tolerance=1e-6,
                                      precision="mixed")
            except Exception as e:  # noqa: BLE001
                err = str(e)
            out["mixed_error"] = err
            assert run.error is None, run.error
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump(out, f)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_plugin_parallel_run_matches_the_whole_mesh_reference(tmp_path):
    import oracle as O
    import torch.multiprocessing as mp
    world = 3
    mp.start_processes(_plugin_rank_main, args=(world, _free_port(), str(tmp_path), "lognormal"),
                       nprocs=world, start_method="spawn")
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    assert all("FP64 only" in (g["mixed_error"] or "") for g in got)
    for name, kind, case in (("cuFoamCG", O.CG, "lognormal"), ("cuFoamBiCG", O.BICG, "convdiff"),
                             ("cuFoamRichardson", O.RICHARDSON, "const")):
        rs = [g[name] for g in got]
        for g in rs[1:]:
            for key in ("k", "final", "init", "conv"):
                assert g[key] == rs[0][key], (name, key)
        L, _, b = _case(case) if case == "lognormal" else _solver_case(case)
        g = rs[0]
        tol = g["tol"]
        want = O.plugin_solve(kind, L, b, np.zeros(L.n), tol, 20000)
        assert g["conv"], name
        assert g["init"] == pytest.approx(want.initial_residual, rel=1e-12)

        class P:
            n_iterations = g["k"]
            final_residual = g["final"]
        assert_fast_order_parity(P, want, reference_band(kind, L, b, np.zeros(L.n), tol, 20000), tol)
        x = np.zeros(L.n)
        for r in rs:
            x[np.array(r["cells"])] = r["x"]
        assert np.linalg.norm(x - want.psi) <= 1e-5 * np.linalg.norm(want.psi)
