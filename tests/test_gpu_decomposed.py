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


def test_decomposed_solve_refuses_other_solvers_and_reports_callback_failures():
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
    with pytest.raises(ConnectionError):
        cf.cuFoamCG("p", A, {"tolerance": 1e-8}, interfaces=ifc).solve(np.zeros(sub.n), np.ones(sub.n))
    with pytest.raises(cf.CufoamError) as e:
        cf.cuFoamBiCG("p", A, {"tolerance": 1e-8}, interfaces=ifc).solve(np.zeros(sub.n), np.ones(sub.n))
    assert e.value.status == 8     # CF_UNSUPPORTED
    A.close()


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
        L, cr, b = _case(case)
        sub = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, cr)[rank]
        psi = np.zeros(sub.n)
        with ParallelRun() as run:
            p = foam_solve_decomposed("cuFoamCG", sub, b[sub.cells], psi, tolerance=TOL, max_iter=MAXIT)
            err = None
            try:   # the other solvers stop with a FatalError in a parallel run
                foam_solve_decomposed("cuFoamBiCG", sub, b[sub.cells], np.zeros(sub.n), tolerance=TOL,
                                      symmetric=False)
            except Exception as e:  # noqa: BLE001
                err = str(e)
            assert run.error is None, run.error
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"k": p["nIterations"], "final": p["finalResidual"], "init": p["initialResidual"],
                       "conv": p["converged"], "cells": sub.cells.tolist(), "x": psi.tolist(),
                       "bicg_error": err}, f)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case,world", [("lognormal", 3)])
def test_plugin_parallel_run_matches_the_whole_mesh_reference(tmp_path, case, world):
    import oracle as O
    import torch.multiprocessing as mp
    mp.start_processes(_plugin_rank_main, args=(world, _free_port(), str(tmp_path), case),
                       nprocs=world, start_method="spawn")
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for g in got[1:]:
        for key in ("k", "final", "init", "conv"):
            assert g[key] == got[0][key], key
    assert all("CG only" in (g["bicg_error"] or "") for g in got)
    L, _, b = _case(case)
    want = O.plugin_solve(O.CG, L, b, np.zeros(L.n), TOL, MAXIT)
    g = got[0]
    assert g["conv"]
    assert g["init"] == pytest.approx(want.initial_residual, rel=1e-12)

    class P:
        n_iterations = g["k"]
        final_residual = g["final"]
    assert_fast_order_parity(P, want, reference_band(O.CG, L, b, np.zeros(L.n), TOL, MAXIT), TOL)
    x = np.zeros(L.n)
    for r in got:
        x[np.array(r["cells"])] = r["x"]
    assert np.linalg.norm(x - want.psi) <= 1e-6 * np.linalg.norm(want.psi)
