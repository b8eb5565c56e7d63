"""Decomposed cases on the CPU: the processor-patch split of an LDU matrix
and the exchange / all-reduce protocol of a decomposed solve, run by two
and three gloo ranks.

OpenFOAM's lduMatrix::Amul on a subdomain is the local product followed
by ``result[faceCells[f]] -= interfaceBouCoeffs[f] * (neighbour's value)``
for every processor face; the sum over subdomains must be the global
product.  The ranks here run CG in numpy through exactly the callbacks the
library calls (``cf_comm`` built by ProcessorComm.as_c), so the host side
of ``cf_solve_decomposed`` is checked without a GPU; the device side is in
test_gpu_decomposed.py."""
import ctypes as C
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from cufoam_gb300 import workloads as W  # noqa: E402
from cufoam_gb300.decomposed import (ProcessorInterfaces, amul_decomposed,  # noqa: E402
                                     decompose)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _global_amul(L, x):
    y = L.diag * x
    np.add.at(y, L.upper_addr, L.lower * x[L.lower_addr])
    np.add.at(y, L.lower_addr, L.upper * x[L.upper_addr])
    return y


def _checker_ranks(nx, ny, nz, n_ranks, block=3):
    """A partition with ragged boundaries: blocks of `block` cells dealt out
    in a pattern, so that some cells have processor faces on several sides
    and to several ranks."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    r = ((i // block) + 2 * (j // block) + (k // block)) % n_ranks
    return r.transpose(2, 1, 0).reshape(-1)   # cell = i + nx (j + ny k)


def _asym(L, seed):
    rng = np.random.default_rng(seed)
    lo = L.lower * (1.0 + 0.3 * rng.random(len(L.lower)))
    up = L.upper * (1.0 + 0.3 * rng.random(len(L.upper)))
    return W.LDU(L.n, L.diag.copy(), lo, up, L.lower_addr, L.upper_addr)


@pytest.mark.parametrize("n_ranks", [2, 3, 5])
def test_subdomain_products_add_up_to_the_global_product(n_ranks):
    L = _asym(W.grid_lognormal(9, 7, 5, 3), 1)
    cr = _checker_ranks(9, 7, 5, n_ranks)
    subs = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, cr)
    x = W.uniform(4, L.n)
    y = _global_amul(L, x)
    owner_of = {}
    for s in subs:
        for p in s.patches:
            for f in p.faces:
                owner_of.setdefault(int(f), []).append(s.rank)
    covered = np.zeros(L.n, bool)
    for s in subs:
        # ghost of face f = the global value of the cell across it
        g = []
        for p in s.patches:
            for f, c in zip(p.faces, p.face_cells):
                gc = s.cells[c]
                other = L.upper_addr[f] if L.lower_addr[f] == gc else L.lower_addr[f]
                g.append(x[other])
        ys = amul_decomposed(s, x[s.cells], np.array(g))
        np.testing.assert_allclose(ys, y[s.cells], rtol=1e-13, atol=1e-13)
        covered[s.cells] = True
        # internal faces stay upper-triangular and sorted by owner
        assert np.all(s.lower_addr < s.upper_addr)
        assert np.all(np.diff(s.lower_addr) >= 0)
    assert covered.all()
    # every processor face appears on exactly its two ranks
    for f, rs in owner_of.items():
        assert sorted(rs) == sorted({int(cr[L.lower_addr[f]]), int(cr[L.upper_addr[f]])})
    # some cell couples to two or more faces (the per-cell face loop is exercised)
    assert any(np.bincount(p.face_cells).max() >= 2 for s in subs for p in s.patches)


def test_patch_faces_are_listed_alike_on_both_sides():
    L = W.grid_const(8, 8, 4)
    subs = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper,
                     _checker_ranks(8, 8, 4, 3, block=2))
    for s in subs:
        for p in s.patches:
            back = [q for q in subs[p.neighbour].patches if q.neighbour == s.rank]
            assert len(back) == 1
            np.testing.assert_array_equal(p.faces, back[0].faces)
            assert np.all(np.diff(p.faces) > 0)
        assert [p.neighbour for p in s.patches] == sorted(p.neighbour for p in s.patches)


def test_decompose_rejects_bad_input():
    L = W.grid_const(4, 4, 1)
    with pytest.raises(ValueError):
        decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, np.zeros(L.n - 1))
    with pytest.raises(ValueError):
        decompose(L.n, L.upper_addr, L.lower_addr, L.diag, L.lower, L.upper, np.zeros(L.n))
    with pytest.raises(ValueError):
        decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper,
                  np.full(L.n, 3), n_ranks=2)


def test_single_rank_has_no_patches():
    L = W.grid_lognormal(6, 5, 4, 2)
    (s,) = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, np.zeros(L.n))
    assert s.patches == [] and s.n == L.n
    np.testing.assert_array_equal(s.lower, L.lower)
    np.testing.assert_array_equal(s.upper_addr, L.upper_addr)


# ---------------------------------------------------------------------------
# the protocol with gloo ranks
# ---------------------------------------------------------------------------
def _cg(apply, dot, b, x, tol, max_iter):
    """CG as the library runs it (SolverSingleGPU.h:366-445): ||r||_2 <= tol."""
    r = b - apply(x)
    rho0 = dot(r, r)
    norm = np.sqrt(rho0)
    hist = [norm]
    k = 0
    rho1 = 0.0
    p = np.zeros_like(b)
    while k < max_iter and norm > tol:
        k += 1
        p = r.copy() if k == 1 else r + (rho0 / rho1) * p
        q = apply(p)
        xi = rho0 / dot(p, q)
        x += xi * p
        r -= xi * q
        rho1 = rho0
        rho0 = dot(r, r)
        norm = np.sqrt(rho0)
        hist.append(norm)
    return k, hist


def _case(name):
    if name == "const":
        return W.grid_const(10, 9, 6), _checker_ranks(10, 9, 6, 2)
    L = W.grid_lognormal(10, 9, 6, 5)
    return L, _checker_ranks(10, 9, 6, 3, block=2)


def _rank_main(rank, world, port, out_dir, case):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        L, cr = _case(case)
        subs = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, cr)
        sub = subs[rank]
        ifc = ProcessorInterfaces.from_subdomain(sub)
        ci, cc = ifc.as_c()
        fc = ifc.face_cells
        b = W.uniform(7, L.n)[sub.cells]
        x = np.zeros(sub.n)

        def apply(v):
            # through the C callback, as the library calls it
            send = np.ascontiguousarray(v[fc]) if ci.n_faces else np.zeros(1)
            recv = np.empty_like(send)
            rc = cc.exchange(None, send.ctypes.data_as(C.POINTER(C.c_double)),
                             recv.ctypes.data_as(C.POINTER(C.c_double)), ci.n_faces)
            assert rc == 0, ifc.comm.error
            return amul_decomposed(sub, v, recv[:ci.n_faces])

        def dot(u, v):
            a = np.array([np.dot(u, v)])
            rc = cc.allreduce_sum(None, a.ctypes.data_as(C.POINTER(C.c_double)), 1)
            assert rc == 0, ifc.comm.error
            return float(a[0])

        k, hist = _cg(apply, dot, b, x, 1e-8, 2000)
        m = np.array([float(rank), -float(rank)])
        rcm = cc.allreduce_max(None, m.ctypes.data_as(C.POINTER(C.c_double)), 2)
        assert rcm == 0 and m.tolist() == [world - 1.0, 0.0], m
        # a wrong count is reported as a failure, not a crash
        bad = np.zeros(2)
        rc = cc.exchange(None, bad.ctypes.data_as(C.POINTER(C.c_double)),
                         bad.ctypes.data_as(C.POINTER(C.c_double)), ci.n_faces + 1)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"k": k, "hist": [float(h) for h in hist], "cells": sub.cells.tolist(),
                       "x": x.tolist(), "bad_rc": int(rc)}, f)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case,world", [("const", 2), ("lognormal", 3)])
def test_decomposed_cg_over_gloo_ranks_matches_the_serial_solve(tmp_path, case, world):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path), case), nprocs=world,
                       start_method="spawn")
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    # every rank took the same decisions on the same (bit-identical) sums
    for g in got[1:]:
        assert g["k"] == got[0]["k"]
        assert g["hist"] == got[0]["hist"]
    assert all(g["bad_rc"] != 0 for g in got)
    L, _ = _case(case)
    b = W.uniform(7, L.n)
    xs = np.zeros(L.n)
    ks, hs = _cg(lambda v: _global_amul(L, v), np.dot, b, xs, 1e-8, 2000)
    x = np.zeros(L.n)
    for g in got:
        x[np.array(g["cells"])] = g["x"]
    assert abs(got[0]["k"] - ks) <= 2, (got[0]["k"], ks)
    np.testing.assert_allclose(got[0]["hist"][0], hs[0], rtol=1e-13)
    assert np.linalg.norm(b - _global_amul(L, x)) <= 1e-8 * 1.0001
    assert np.linalg.norm(x - xs) <= 1e-6 * np.linalg.norm(xs)


# ---------------------------------------------------------------------------
# the OpenFOAM plugin's processor-patch callbacks (cuFoamGB300Comm.H) over
# the stand-in's Pstream, carried by gloo
# ---------------------------------------------------------------------------
def _plugin_rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from cufoam_gb300.plugin import ParallelRun, processor_comm_check
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        L = W.grid_lognormal(8, 7, 6, 2)
        cr = _checker_ranks(8, 7, 6, world, block=2)
        sub = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper, cr)[rank]
        x = W.uniform(3, L.n)
        fc, _ = sub.interface_arrays()
        vals = np.array([rank + 0.5, 1e-3 * (rank + 1), -2.0 * rank])
        with ParallelRun() as run:
            rc, recv, summed, maxed = processor_comm_check(sub, x[sub.cells][fc], vals)
            assert run.error is None, run.error
            # a second round through the same patches
            rc2, recv2, _, _ = processor_comm_check(sub, 2.0 * x[sub.cells][fc], vals)
        want = []
        for p in sub.patches:
            for f, c in zip(p.faces, p.face_cells):
                g = sub.cells[c]
                want.append(x[L.upper_addr[f] if L.lower_addr[f] == g else L.lower_addr[f]])
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"rc": [rc, rc2], "recv_ok": bool(np.array_equal(recv, np.array(want))),
                       "recv2_ok": bool(np.array_equal(recv2, 2.0 * np.array(want))),
                       "summed": summed.tolist(), "maxed": maxed.tolist(), "n": int(len(fc))}, f)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_plugin_processor_callbacks_over_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 3
    mp.start_processes(_plugin_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn")
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    want = np.zeros(3)
    vals = [np.array([r + 0.5, 1e-3 * (r + 1), -2.0 * r]) for r in range(world)]
    for v in vals:
        want += v
    for g in got:
        assert g["rc"] == [0, 0]
        assert g["n"] > 0 and g["recv_ok"] and g["recv2_ok"]
        assert g["summed"] == got[0]["summed"]
        assert g["maxed"] == np.max(vals, axis=0).tolist()
    np.testing.assert_allclose(got[0]["summed"], want, rtol=1e-15)


def test_plugin_refuses_processor_patches_outside_a_parallel_run():
    # the solver stops before it touches the GPU
    from cufoam_gb300.plugin import FoamError, foam_solve, processor_comm_check
    L = W.grid_const(4, 4, 2)
    with pytest.raises(FoamError, match="outside a parallel run"):
        foam_solve("cuFoamCG", L, W.uniform(1, L.n), np.zeros(L.n), processor_patch=True)
    # and the stand-in's Pstream moves nothing in a serial run: the
    # callbacks report the failure
    sub = decompose(L.n, L.lower_addr, L.upper_addr, L.diag, L.lower, L.upper,
                    (np.arange(L.n) % 2))[0]
    fc, _ = sub.interface_arrays()
    rc, _, _, _ = processor_comm_check(sub, np.zeros(len(fc)), np.zeros(1))
    assert rc == 1


def _two_patch_rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from cufoam_gb300.decomposed import ProcessorComm, ProcessorPatch
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        other = 1 - rank
        # two patches between the same two ranks (as a processorCyclic patch
        # beside a plain processor patch), of different sizes
        patches = [ProcessorPatch(other, np.array([0, 1, 2], np.int32), np.ones(3), np.arange(3)),
                   ProcessorPatch(other, np.array([3, 4], np.int32), np.ones(2), np.arange(3, 5))]
        comm = ProcessorComm(patches)
        send = 10.0 * rank + np.arange(5, dtype=np.float64)
        recv = np.zeros(5)
        comm.exchange(send, recv)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"recv": recv.tolist()}, f)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_patches_to_one_neighbour_are_kept_apart(tmp_path):
    import torch.multiprocessing as mp
    mp.start_processes(_two_patch_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2,
                       start_method="spawn")
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert got[0]["recv"] == [10.0, 11.0, 12.0, 13.0, 14.0]
    assert got[1]["recv"] == [0.0, 1.0, 2.0, 3.0, 4.0]
