#!/usr/bin/env python3
"""Benchmark of the sparse solve path on one workload:

    3-D 7-point Poisson, 128^3 cells (2,097,152 rows, 14,581,760 nnz), FP64
    LDU form (diag 6, off-diagonals -1, Dirichlet walls folded), seeded
    uniform[-1,1] source, psi0 = 0, solved by the cuFoamCG plugin at
    tolerance 1e-8 (relative to normFactor).

A step is one complete solve.  `value` is the solve's algorithmic HBM
traffic (bytes every kernel of the fused schedule must move, see
`solve_bytes`) divided by the device time, with the matrix and vectors
resident in HBM (inputs exceed L2, so no flush is needed).  `e2e` is the
same metric through the public API with host buffers, as the plugin runs a
time step on a mesh it has seen: every step uploads the new LDU
coefficients from pinned host memory into the cached device matrix
(refreshing its CSR and SELL-32 values on the device), solves with host
psi/source and reads psi back; `e2e.first_call` adds the addressing upload
and the device ldu2csr / SELL-32 build of a new mesh.  `--impl reference` times the CPU restatement of the reference's CG
(the oracle, all host threads) on bounded samples of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX = NY = NZ = 128
TOL = 1e-8
MAX_ITER = 10000
SEED = 3
WORKLOAD = "poisson7_128^3_fp64_cuFoamCG_tol1e-8"


# ---------------------------------------------------------------------------
# algorithmic bytes of the fused CG schedule (FP64 values, int32 indices)
# ---------------------------------------------------------------------------
# The iteration kernels stream the matrix in the format the library picked
# for it (SELL-32 with one-byte column codes for this stencil: 9 B per
# stored entry incl. padding, one int32 offset per 32-row slice, a 128 B
# offset table; 12 B per entry with 32-bit columns); the set-up kernels read
# the CSR arrays.
# Every figure below counts each vector a kernel touches once.
def csr_matrix_bytes(n: int, nnz: int) -> int:
    return 12 * nnz + 4 * (n + 1)


def sell_matrix_bytes(n: int, stored: int) -> int:
    return 12 * stored + 4 * ((n + 31) // 32 + 1)


def sell8_matrix_bytes(n: int, stored: int) -> int:
    """SELL-32 with one-byte column codes: 8 B value + 1 B code per stored
    entry, one int32 offset per slice, the 32-entry offset table."""
    return 9 * stored + 4 * ((n + 31) // 32 + 1) + 4 * 32


def sell16_matrix_bytes(n: int, stored: int) -> int:
    """SELL-32 with 16-bit column deltas: 8 B value + 2 B delta per stored
    entry, one int32 offset per slice."""
    return 10 * stored + 4 * ((n + 31) // 32 + 1)


def iter_matrix_bytes(fmt: str, n: int, nnz: int, stored: int, fp64_loop: bool = False) -> int:
    """FP64 matrix bytes per pass of the fast kernels in the format in use.
    fp64_loop: a pass of an FP64 solver loop, which reads the 32-bit columns
    when the codes exist by default (the codes serve the plain product and
    the FP32 sweeps)."""
    if fmt in ("sell8", "sell16") and fp64_loop:
        fmt = "sell"
    if fmt == "sell16":
        return sell16_matrix_bytes(n, stored)
    if fmt == "sell8":
        return sell8_matrix_bytes(n, stored)
    if fmt == "sell":
        return sell_matrix_bytes(n, stored)
    return csr_matrix_bytes(n, nnz)


def spmv_bytes(mat: int, n: int) -> int:
    """SpMV compulsory traffic: the matrix, x once, y written."""
    return mat + 8 * n + 8 * n


def cg_iteration_bytes(mat: int, n: int) -> int:
    """One CG step of the default schedule: prep (r, p, x read; p, x
    written), spmv (q = A p; p gathered, counted once), update (q, r read;
    r written)."""
    return 40 * n + spmv_bytes(mat, n) + 24 * n


def solve_bytes(mat_iter: int, mat_csr: int, n: int, iters: int) -> int:
    setup = 8 * n + (mat_csr + 16 * n) + (mat_csr + 24 * n)     # nf_sum, nf_dist, res_init
    per_iter = cg_iteration_bytes(mat_iter, n)
    first = per_iter - 24 * n                                     # step 1: p = r, no x update
    flush = 24 * n
    if iters == 0:
        return setup
    return setup + first + (iters - 1) * per_iter + flush


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profiled_value(name: str, key: str):
    """A `key: value` line of a committed ncu summary (profiles/<name>),
    or None."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def profiled_traffic(name: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary, or None."""
    v = profiled_value(name, "traffic_bytes_per_launch")
    return None if v is None else int(v)


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_problem():
    from cufoam_gb300 import workloads as W
    L = W.grid_const(NX, NY, NZ)
    b = W.uniform(SEED, L.n)
    return L, b


def cpu_baseline(L, b, iters: int):
    """The oracle's reference-order CG (OpenMP, all host threads) for a
    bounded number of iterations; returns (GB/s, cores, seconds)."""
    import oracle as O
    A = O.ldu2csr(L)
    x0 = np.zeros(L.n)
    O.solve(O.CG, A, b, x0, 0.0, 2)  # warm-up: page in, spin up threads
    t0 = time.perf_counter()
    r = O.solve(O.CG, A, b, x0, 0.0, iters)
    dt = time.perf_counter() - t0
    nf_time_share = 0  # normFactor is not part of the sample
    del nf_time_share
    mat = csr_matrix_bytes(A.n, A.nnz)
    bytes_ = (mat + 24 * A.n) + r.n_iterations * cg_iteration_bytes(mat, A.n)
    return bytes_ / dt / 1e9, O.get_threads(), dt, r.n_iterations


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    L, b = make_problem()
    import oracle as O
    A = O.ldu2csr(L)
    x0 = np.zeros(L.n)
    sample = 20
    for _ in range(args.warmup):
        O.solve(O.CG, A, b, x0, 0.0, sample)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.solve(O.CG, A, b, x0, 0.0, sample)
        times.append(time.perf_counter() - t0)
    mat = csr_matrix_bytes(A.n, A.nnz)
    bytes_step = (mat + 24 * A.n) + sample * cg_iteration_bytes(mat, A.n)
    total = sum(times)
    value = bytes_step * args.steps / total / 1e9
    cores = O.get_threads()
    # the same sample on one host core
    O.set_threads(1)
    try:
        t0 = time.perf_counter()
        O.solve(O.CG, A, b, x0, 0.0, sample)
        one_core = bytes_step / (time.perf_counter() - t0) / 1e9
    finally:
        O.set_threads(cores)
    line = {
        "metric": "solve_hbm_gbs", "value": round(value, 3), "unit": "GB/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rows": L.n, "nnz": A.nnz},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} CG iterations of the 128^3 solve per step "
                                   f"(plain-C restatement of SolverSingleGPU.h CG, OpenMP)",
                         "cpu_model": host_cpu_model(), "one_core_gbs": round(one_core, 3)},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "cpu_one_core": {"value": round(one_core, 3), "unit": "GB/s", "cores": 1},
        "reference_gpu_kernels": reference_gpu_cg(A, b),
    }
    print(json.dumps(line))
    return 0


def reference_gpu_cg(A, b):
    """The whole 128^3 CG solve through the reference's own kernels on this
    GPU (gis/SparseSystem/kernels.h compiled from the reference sources into
    oracle/_ref/ref_kernels.cubin) with its host loop (SolverSingleGPU.h
    CG: two synchronous host-summed dot products and their allocations per
    step), matrix and vectors already on the device.  Rate in the same
    algorithmic bytes as the `solve_hbm_gbs` line of this build."""
    import oracle as O
    try:
        import torch
        if not torch.cuda.is_available() or not O.reference_kernels.available():
            return {"unavailable": "no GPU or no compiled reference kernels"}
        x0 = np.zeros(A.n)
        nf = O.norm_factor(A, b, x0)
        with O.reference_kernels(0) as rk:
            rk.cg_device(A, b, x0, 0.0, 3)
            _, _, k, ms = rk.cg_device(A, b, x0, TOL * nf, MAX_ITER)
        mat = csr_matrix_bytes(A.n, A.nnz)
        work = (mat + 24 * A.n) + k * cg_iteration_bytes(mat, A.n)
        return {"ms_per_solve": round(ms, 2), "iterations": k, "value": round(work / (ms * 1e-3) / 1e9, 2),
                "unit": "GB/s", "path": "reference kernels + reference host loop, device-resident data"}
    except Exception as e:  # informative only, never fatal to the line
        return {"unavailable": repr(e)}


def host_cpu_model() -> str:
    """The host CPU's model name (lscpu / /proc/cpuinfo), or "unknown"."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


# algorithmic bytes per step of the other fast-order schedules (FP64 values,
# int32 indices; `mat` = the streamed matrix bytes; each vector a kernel
# touches counted once): Jacobi one pass over A D^-1 (matrix + r gathered,
# r written, x and 1/a_ii read, x written); Richardson prep (r, x read, x
# written) + residual pass (matrix + x gathered, b read, r written)
def jacobi_step_bytes(mat: int, n: int) -> int:
    return mat + 8 * n * 5


def richardson_step_bytes(mat: int, n: int) -> int:
    return 24 * n + mat + 8 * n * 3


def timed_solve(solver_cls, M, src, ctrl, dev):
    """One solve on device vectors after a short warm-up solve (graphs,
    scaled copies): (perf, wall seconds)."""
    import torch
    psi = torch.zeros(M.n, dtype=torch.float64, device=dev)
    solver_cls("p", M, dict(ctrl, maxIter=8)).solve(psi, src)
    psi.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    perf = solver_cls("p", M, ctrl).solve(psi, src)
    torch.cuda.synchronize()
    return perf, time.perf_counter() - t0


def suite_c1(ctx, device):
    """C1: the 64x64 5-point Poisson system (4,096 rows), tolerance 1e-6 --
    latency, not bandwidth (the whole system sits in L2): device time per
    solver step for CG, Jacobi and Richardson, and the device ldu2csr."""
    import ctypes as C

    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import _capi
    from cufoam_gb300 import workloads as W
    dev = f"cuda:{device}"
    L = W.grid_const(64, 64, 1)
    src = torch.from_numpy(W.uniform(1, L.n)).to(dev)
    M = cf.LduMatrix.from_ldu(L, ctx)
    out = {}
    for name, key in (("cuFoamCG", "cg"), ("cuFoamJacobi", "jacobi"), ("cuFoamRichardson", "richardson")):
        perf, _ = timed_solve(cf._TABLE[name], M, src, {"tolerance": 1e-6, "maxIter": 1000000}, dev)
        out[key] = {"iters": perf.n_iterations, "ms": round(perf.solve_ms, 3),
                    "us_per_step": round(1e3 * perf.solve_ms / max(perf.n_iterations, 1), 2),
                    "status": perf.status_name}
    M.close()
    # device ldu2csr of the same mesh: LDU arrays on the device, CSR into
    # device buffers (cf_ldu2csr), wall time per conversion
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(L, k))).to(dev)
         for k in ("diag", "lower", "upper", "lower_addr", "upper_addr")}
    v, keep = cf._ldu_view(L.n, t["diag"], t["lower"], t["upper"], t["lower_addr"], t["upper_addr"])
    nnz = L.n + 2 * t["lower"].shape[0]
    ro = torch.empty(L.n + 1, dtype=torch.int32, device=dev)
    co = torch.empty(nnz, dtype=torch.int32, device=dev)
    va = torch.empty(nnz, dtype=torch.float64, device=dev)
    lib = _capi.load()
    ctx.set_stream(torch.cuda.current_stream(device))

    def conv():
        ctx.check(lib.cf_ldu2csr(ctx.handle, C.byref(v), ro.data_ptr(), co.data_ptr(), va.data_ptr(),
                                 _capi.CF_MEM_DEVICE), "cf_ldu2csr")
    for _ in range(3):
        conv()
    torch.cuda.synchronize()
    reps = 50
    t0 = time.perf_counter()
    for _ in range(reps):
        conv()
    torch.cuda.synchronize()
    out["ldu2csr_us"] = round(1e6 * (time.perf_counter() - t0) / reps, 2)
    del keep
    return out


def suite_c2(ctx, device):
    """C2: 7-point Poisson at 128^3, constant and lognormal(0,1) coefficients,
    tolerance 1e-8 through the plugin path (default summation order): CG,
    Jacobi and Richardson -- time, steps, algorithmic GB/s.  Richardson
    diverges on the lognormal system in the reference algorithm itself (its
    30-step power method underestimates the largest eigenvalue there), and
    here too, at the same step."""
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    dev = f"cuda:{device}"
    src = torch.from_numpy(W.uniform(3, NX * NY * NZ)).to(dev)
    out = {}
    for case, make in (("const", lambda: W.grid_const(NX, NY, NZ)),
                       ("lognormal", lambda: W.grid_lognormal(NX, NY, NZ, 2))):
        L = make()
        M = cf.LduMatrix.from_ldu(L, ctx)
        n, _, nnz = M.shape()
        fmt, stored = M.format()
        mat = iter_matrix_bytes(fmt, n, nnz, stored, fp64_loop=True)
        res = {}
        for name, key, per in (("cuFoamCG", "cg", cg_iteration_bytes),
                               ("cuFoamJacobi", "jacobi", jacobi_step_bytes),
                               ("cuFoamRichardson", "richardson", richardson_step_bytes)):
            if case == "const" and key == "cg":
                continue                                  # the headline line
            perf, _ = timed_solve(cf._TABLE[name], M, src, {"tolerance": TOL, "maxIter": 400000}, dev)
            k = perf.n_iterations
            res[key] = {"iters": k, "ms": round(perf.solve_ms, 2), "status": perf.status_name,
                        "gbs": round(per(mat, n) * k / (perf.solve_ms * 1e-3) / 1e9, 1)}
        if case == "const":
            # CG in FP64 and in mixed precision (FP32 sweeps over the one-byte
            # column codes, FP64 refinement) to the same tolerance; the time
            # and the true relative residual ||b - A x|| / normFactor of each
            mx = {}
            for prec in ("FP64", "mixed"):
                psi = torch.zeros(n, dtype=torch.float64, device=dev)
                c = {"tolerance": TOL, "maxIter": 400000, "precision": prec}
                cf.cuFoamCG("p", M, dict(c, maxIter=8)).solve(psi, src)
                psi.zero_()
                torch.cuda.synchronize()
                perf = cf.cuFoamCG("p", M, c).solve(psi, src)
                torch.cuda.synchronize()
                r = src - M.spmv(psi, row_order="fast")
                mx[prec] = {"ms": round(perf.solve_ms, 2), "iters": perf.n_iterations, "status": perf.status_name,
                            "true": float(f"{float(torch.linalg.norm(r)) / perf.norm_factor:.3g}")}
            mx["speedup"] = round(mx["FP64"]["ms"] / mx["mixed"]["ms"], 3)
            out["cg_mixed_vs_fp64"] = mx
        out[case] = res
        M.close()
    return out


def suite_c5(ctx, device, n: int = 96, tol: float = 1e-10):
    """C5: the differentiable diffusion solve at 96^3 (face conductivity
    exp(g), g a Gaussian random field of correlation length 8 cells; loss
    0.5 ||x - x_t||^2): forward CG solve and backward pass (adjoint CG solve
    of A^T lambda = x - x_t plus the gradient scatter), wall time with the
    device synchronised, tolerance 1e-10."""
    import torch

    from cufoam_gb300 import workloads as W
    from cufoam_gb300.autograd import LduPattern, ldu_solve
    dev = f"cuda:{device}"
    g = W.grid_grf(n, n, n, 5, 8.0)
    L, kf, kb = W.diffusion_from_cells(n, n, n, g)
    b = torch.from_numpy(W.uniform(6, L.n)).to(dev)
    xt = torch.from_numpy(0.05 * np.cos(np.linspace(0, 6.0, L.n))).to(dev)
    la = torch.from_numpy(L.lower_addr.astype(np.int64)).to(dev)
    ua = torch.from_numpy(L.upper_addr.astype(np.int64)).to(dev)
    kf_t = torch.from_numpy(kf).to(dev).requires_grad_(True)
    kb_t = torch.from_numpy(kb).to(dev)
    pattern = LduPattern(L.n, L.lower_addr, L.upper_addr, context=ctx)

    def fwd():
        diag = kb_t.index_add(0, la, kf_t).index_add(0, ua, kf_t)
        x = ldu_solve(diag, -kf_t, -kf_t, b, pattern, {"tolerance": tol, "maxIter": 100000})
        return 0.5 * ((x - xt) ** 2).sum()
    loss = fwd()
    loss.backward()                       # warm-up: matrix, transpose, graphs
    kf_t.grad = None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = fwd()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    loss.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return {"rows": L.n, "forward_ms": round(1e3 * (t1 - t0), 2), "backward_ms": round(1e3 * (t2 - t1), 2),
            "tolerance": tol, "grad_norm": float(torch.linalg.norm(kf_t.grad))}


def compact_suite(extras: dict) -> dict:
    """The figures of the other configurations, short enough for the one
    JSON line: C1 latency, C2 solvers, C3 mixed vs FP64, C4 batched vs
    sequential, C5 forward + backward."""
    out = {}
    c1 = extras.get("c1")
    if isinstance(c1, dict) and "error" not in c1:
        out["c1_64^2_us_per_step"] = {k: c1[k]["us_per_step"] for k in ("cg", "jacobi", "richardson")}
        out["c1_iters"] = {k: c1[k]["iters"] for k in ("cg", "jacobi", "richardson")}
        out["c1_ldu2csr_us"] = c1["ldu2csr_us"]
    c2 = extras.get("c2")
    if isinstance(c2, dict) and "error" not in c2:
        if "cg_mixed_vs_fp64" in c2:
            out["c2_const_cg_mixed_vs_fp64"] = c2["cg_mixed_vs_fp64"]
        for case, res in c2.items():
            if case == "cg_mixed_vs_fp64":
                continue
            for k, r in res.items():
                out[f"c2_{case}_{k}"] = {"iters": r["iters"], "ms": r["ms"], "gbs": r["gbs"],
                                         "status": r["status"]}
    for key, short in (("mixed_vs_fp64", "c3_mr"), ("mixed_vs_fp64_mrjacobi", "c3_mrjacobi"),
                       ("mixed_vs_fp64_bicg", "c3_bicg_pe10"), ("mixed_vs_fp64_bicg_pe1", "c3_bicg_pe1")):
        r = extras.get(key)
        if isinstance(r, dict) and "FP64" in r:
            f, m = r["FP64"], r["mixed"]
            out[short] = {"fp64_ms": f["ms"], "fp64_it": f["iterations"], "fp64_status": f["status"],
                          "fp64_true": float(f"{f['true_rel_residual']:.3g}"),
                          "mixed_ms": m["ms"], "mixed_it": m["iterations"], "mixed_status": m["status"],
                          "mixed_true": float(f"{m['true_rel_residual']:.3g}"),
                          "speedup": r["speedup"],
                          "err_vs_fp64": float(f"{m['rel_error_vs_fp64']:.3g}")}
            for arm, k in (("FP64", "fp64_tightened_tol"), ("mixed", "mixed_tightened_tol")):
                if "tightened_tolerance" in r[arm]:
                    out[short][k] = float(f"{r[arm]['tightened_tolerance']:.3g}")
            if "FP64_fast" in r:
                ff = r["FP64_fast"]
                out[short].update({"fp64_fast_ms": ff["ms"], "fp64_fast_it": ff["iterations"],
                                   "fp64_fast_status": ff["status"],
                                   "fp64_fast_true": float(f"{ff['true_rel_residual']:.3g}"),
                                   "speedup_vs_fp64_fast": r.get("speedup_vs_fast")})
    r = extras.get("batched_vs_sequential")
    if isinstance(r, dict) and "batched_ms" in r:
        out["c4"] = {"batched_ms": r["batched_ms"], "sequential_ms": r["sequential_ms"],
                     "speedup": r["speedup"], "converged": r["batched_converged"],
                     "mixed_ms": r["mixed"]["batched_ms"],
                     "mixed_speedup_vs_seq": r["mixed"]["speedup_vs_sequential_fp64"]}
    r = extras.get("c5")
    if isinstance(r, dict) and "forward_ms" in r:
        out["c5_96^3_ms"] = {"forward": r["forward_ms"], "backward": r["backward_ms"]}
    errs = {k: v["error"][:80] for k, v in extras.items() if isinstance(v, dict) and "error" in v}
    if errs:
        out["errors"] = errs
    return out


def max_over_ranks(value: float, dist, device: str) -> float:
    """The largest of every rank's `value` (the job's time is its slowest
    rank's); the value itself without a process group."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist, device: str) -> float:
    """The sum of every rank's `value` (work done by the whole job)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_ours(args):
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if world > 1 else 0
    torch.cuda.set_device(device)

    L, b = make_problem()
    ctx = cf.Context(device)
    stream = torch.cuda.current_stream(device)
    ctx.set_stream(stream)
    M = cf.LduMatrix.from_ldu(L, ctx)
    n, nf, nnz = M.shape()
    fmt, stored = M.format()
    mat_csr = csr_matrix_bytes(n, nnz)
    mat_it = iter_matrix_bytes(fmt, n, nnz, stored, fp64_loop=True)    # the CG loop's passes
    mat_spmv = iter_matrix_bytes(fmt, n, nnz, stored)                  # the plain product
    src = torch.from_numpy(b).to(f"cuda:{device}")
    psi = torch.zeros(n, dtype=torch.float64, device=f"cuda:{device}")
    solver = cf.cuFoamCG("p", M, {"tolerance": TOL, "maxIter": MAX_ITER})

    def step():
        psi.zero_()
        return solver.solve(psi, src)

    for _ in range(max(args.warmup, 3)):
        perf = step()
    iters = perf.n_iterations
    torch.cuda.synchronize()

    clocks = ClockSampler(device)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    its = []
    for _ in range(args.steps):
        its.append(step().n_iterations)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clock_info = clocks.stop()
    dev = f"cuda:{device}"
    ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    # replicas: every rank solves its own copy; the job's work is the sum
    bytes_total = sum_over_ranks(sum(solve_bytes(mat_it, mat_csr, n, k) for k in its), dist, dev)
    csr_equiv = sum_over_ranks(sum(solve_bytes(mat_csr, mat_csr, n, k) for k in its), dist, dev)
    value = bytes_total / (ms * 1e-3) / 1e9
    # nf_sum, nf_dist, res_init, flush, clear, and 3 kernels per step in
    # passes of 8 steps (the steps of the last pass past convergence return
    # at once)
    launches = sum(5 + 3 * 8 * ((k + 7) // 8) for k in its)

    # ---- e2e through the public API with pinned host buffers -------------
    # What the plugin does per cuFoamCG::solve in a running case (its device
    # matrix is cached per mesh addressing, plugin/cuFoamGB300.C
    # deviceMatrix()): upload the new coefficients, upload source and psi,
    # solve, download psi.  The first call on a mesh also uploads the
    # addressing and builds the CSR and SELL-32 copies: timed separately
    # as `first_call`.
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    h = {k: pin(getattr(L, k)) for k in ("diag", "lower", "upper", "lower_addr", "upper_addr")}
    hb = pin(b)
    hpsi = pin(np.zeros(n))
    h2d_first = sum(v.nbytes for v in h.values()) + hb.nbytes + hpsi.nbytes
    h2d = h["diag"].nbytes + h["lower"].nbytes + h["upper"].nbytes + hb.nbytes + hpsi.nbytes
    d2h = hpsi.nbytes
    ctrl = {"tolerance": TOL, "maxIter": MAX_ITER}

    def first_call():
        hpsi[:] = 0.0
        m = cf.LduMatrix(L.n, h["diag"], h["lower"], h["upper"], h["lower_addr"],
                         h["upper_addr"], context=ctx)
        p = cf.cuFoamCG("p", m, ctrl).solve(hpsi, hb)
        m.close()
        return p

    m_e2e = cf.LduMatrix(L.n, h["diag"], h["lower"], h["upper"], h["lower_addr"], h["upper_addr"],
                         context=ctx)

    def e2e_step():
        hpsi[:] = 0.0
        m_e2e.update_values(h["diag"], h["lower"], h["upper"])
        return cf.cuFoamCG("p", m_e2e, ctrl).solve(hpsi, hb)

    for _ in range(max(args.warmup, 3)):
        e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e_its = [e2e_step().n_iterations for _ in range(max(1, args.steps))]
    e_dt = max_over_ranks(time.perf_counter() - t0, dist, f"cuda:{device}")
    e2e_value = sum_over_ranks(sum(solve_bytes(mat_it, mat_csr, n, k) for k in e_its), dist,
                               f"cuda:{device}") / e_dt / 1e9
    first_call()
    t0 = time.perf_counter()
    f_its = first_call().n_iterations
    f_dt = time.perf_counter() - t0
    m_e2e.close()

    # ---- dominant kernel: per-launch time with CUDA events (profiled solve)
    psi.zero_()
    prof = cf.cuFoamCG("p", M, {"tolerance": TOL, "maxIter": MAX_ITER,
                                "profileKernels": 1})
    pp = prof.solve(psi, src)
    k1_ms = pp.kernel_ms[0] / max(pp.kernel_launches[0], 1)
    k2_ms = pp.kernel_ms[1] / max(pp.kernel_launches[1], 1)
    k0_ms = pp.kernel_ms[2] / max(pp.kernel_launches[2], 1)
    peak, peak_kind = measured_hbm_peak()
    k1_bytes = spmv_bytes(mat_it, n)
    k1_gbs = k1_bytes / (k1_ms * 1e-3) / 1e9
    k2_gbs = 24 * n / (k2_ms * 1e-3) / 1e9
    k0_gbs = 40 * n / (k0_ms * 1e-3) / 1e9

    # ---- plain SpMV (y = A x) with CUDA events ---------------------------
    x = torch.from_numpy(W.uniform(5, n)).to(f"cuda:{device}")
    y = torch.empty_like(x)

    def time_spmv(reps=50):
        for _ in range(3):
            M.spmv(x, row_order="fast", out=y)
        torch.cuda.synchronize()
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        for _ in range(reps):
            M.spmv(x, row_order="fast", out=y)   # enqueued back to back on the stream
        s1.record(stream)
        torch.cuda.synchronize()
        return s0.elapsed_time(s1) / reps

    # the product in the format AUTO picks (one-byte column codes here), and
    # over the 32-bit columns of the SELL-32 copy (the CG loop's format)
    spmv_c8_ms = time_spmv()
    spmv_c8_gbs = spmv_bytes(mat_spmv, n) / (spmv_c8_ms * 1e-3) / 1e9
    spmv_ms, spmv_gbs = spmv_c8_ms, spmv_c8_gbs
    if fmt == "sell8":
        M.set_format("sell")
        spmv_ms = time_spmv()
        spmv_gbs = spmv_bytes(sell_matrix_bytes(n, stored), n) / (spmv_ms * 1e-3) / 1e9
        M.set_format("auto")
        M.format()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    extras = {}
    if world == 1 and not args.no_extras:
        # C3 (cell Peclet 10): MR and MRJacobi converge in both precisions;
        # FP64 BiCG does not reach 1e-10 there in either summation order
        # while mixed BiCG (FP32 BiCGStab sweeps) converges; at cell Peclet 1
        # FP64 BiCG converges and the times compare
        for key, solver, mx, pe in (("mixed_vs_fp64", "cuFoamMR", 100000, 10.0),
                                    ("mixed_vs_fp64_mrjacobi", "cuFoamMRJacobi", 100000, 10.0),
                                    ("mixed_vs_fp64_bicg", "cuFoamBiCG", 4000, 10.0),
                                    ("mixed_vs_fp64_bicg_pe1", "cuFoamBiCG", 20000, 1.0)):
            try:
                extras[key] = mixed_vs_fp64(ctx, device, solver, pe=pe, max_iter=mx)
            except Exception as e:  # reported, never fatal to the headline line
                extras[key] = {"error": repr(e)}
        for key, fn in (("batched_vs_sequential", batched_vs_sequential), ("c1", suite_c1),
                        ("c2", suite_c2), ("c5", suite_c5)):
            try:
                extras[key] = fn(ctx, device)
            except Exception as e:
                extras[key] = {"error": repr(e)}

    base_gbs, cores, base_dt, base_it = cpu_baseline(L, b, 40)
    import oracle as O
    O.set_threads(1)
    try:
        one_gbs = cpu_baseline(L, b, 10)[0]
    finally:
        O.set_threads(cores)
    line = {
        "metric": "solve_hbm_gbs", "value": round(value, 2), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rows": n, "nnz": nnz, "faces": nf,
                   "iterations": iters, "tolerance": TOL, "reduction": "auto (fast for CG)",
                   "spmv_format": fmt, "cg_loop_format": "sell" if fmt == "sell8" else fmt,
                   "stored_entries": stored,
                   "l2": f"inputs larger than L2 ({spmv_bytes(mat_it, n) / 1e6:.1f} MB per SpMV "
                         f"pass vs 129 MB L2)",
                   "parallelism": f"replicas x{world}",
                   "csr_equivalent_gbs": round(csr_equiv / (ms * 1e-3) / 1e9, 2),
                   "suite": compact_suite(extras)},
        "e2e": {"value": round(e2e_value, 2), "unit": "GB/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "ms_per_step": round(1e3 * e_dt / len(e_its), 3),
                "path": "cuFoamCG.solve with host arrays on the cached device matrix: "
                        "coefficient, source and psi upload, solve, psi download",
                "first_call": {"ms": round(1e3 * f_dt, 3), "h2d_bytes": int(h2d_first),
                               "value": round(solve_bytes(mat_it, mat_csr, n, f_its) / f_dt / 1e9, 2),
                               "path": "a new mesh: addressing upload, device ldu2csr and "
                                       "SELL-32 build, then the solve"}},
        "roofline": {"bound": "hbm", "kernel": "k_f_cg_spmv", "achieved": round(k1_gbs, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(k1_gbs / peak, 4),
                     "peak_source": peak_kind,
                     "bytes_per_launch": k1_bytes,
                     "us_per_launch": round(k1_ms * 1e3, 2),
                     "traffic": profiled_traffic("k_f_cg_spmv_sell_poisson128.md"),
                     # the co-binding unit: 8 FP64 operations per row (ncu, same summary)
                     "fp64_pipe_active": profiled_value("k_f_cg_spmv_sell_poisson128.md",
                                                        "fp64_pipe_active_frac"),
                     # the plain SpMV y = A x (cf_spmv_async, back to back)
                     "spmv_us": round(spmv_ms * 1e3, 2), "spmv_gbs": round(spmv_gbs, 1),
                     "spmv_frac": round(spmv_gbs / peak, 4),
                     # the same product over the one-byte column codes (9 B per entry)
                     "spmv_c8_us": round(spmv_c8_ms * 1e3, 2), "spmv_c8_gbs": round(spmv_c8_gbs, 1),
                     "spmv_c8_frac": round(spmv_c8_gbs / peak, 4),
                     # the other two kernels of the CG step, CUDA events per launch
                     "cg_update_us": round(k2_ms * 1e3, 2), "cg_update_gbs": round(k2_gbs, 1),
                     "cg_prep_us": round(k0_ms * 1e3, 2), "cg_prep_gbs": round(k0_gbs, 1),
                     "cg_step_us": round(1e3 * ms / args.steps / max(iters, 1), 2)},
        "cpu_baseline": {"value": round(base_gbs, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": f"{base_it} CG iterations on the same 128^3 system "
                                   f"({base_dt:.1f} s, oracle restatement, OpenMP)",
                         "cpu_model": host_cpu_model(), "one_core_gbs": round(one_gbs, 3)},
        "gpu_launches": int(launches),
        "clocks": clock_info,
    }
    if extras:
        # the full comparison records go to stderr; the line keeps the
        # compact figures (config.suite)
        print(json.dumps({"details": extras}), file=sys.stderr, flush=True)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def mixed_vs_fp64(ctx, device, solver: str = "cuFoamMR", n: int = 256, pe: float = 10.0,
                  tol: float = 1e-10, max_iter: int = 100000):
    """One solver on the n^3 upwind convection-diffusion system (cell Peclet
    up to pe): the plain FP64 solve vs the mixed-precision solve (FP32 inner
    solver, FP64 residual / normFactor / refinement) to the same FP64
    relative residual; the mixed answer's error against the FP64 one."""
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    t0 = time.perf_counter()
    L, stats = W.grid_convdiff(n, n, n, 7, pe)
    b = W.uniform(8, L.n)
    gen_s = time.perf_counter() - t0
    M = cf.LduMatrix.from_ldu(L, ctx)
    dev = f"cuda:{device}"
    src = torch.from_numpy(b).to(dev)
    out = {"workload": f"convdiff7_upwind_{n}^3_pe{stats['pe_max']:g}_{solver}", "rows": L.n,
           "nnz": M.shape()[2], "tolerance": tol, "max_iter": max_iter, "generate_s": round(gen_s, 1)}
    res = {}
    # BiCG's default FP64 order is the reference's; its fast order is timed too
    arms = ("FP64", "mixed", "FP64_fast") if solver == "cuFoamBiCG" else ("FP64", "mixed")
    for prec in arms:
        ctrl = {"tolerance": tol, "maxIter": max_iter, "precision": prec.split("_")[0],
                "maxRefinements": 200}
        if prec == "FP64_fast":
            ctrl["reduction"] = "fast"
        psi = torch.zeros(L.n, dtype=torch.float64, device=dev)
        cf._TABLE[solver]("U", M, dict(ctrl, maxIter=5)).solve(psi, src)  # warm-up: graphs, FP32 copy
        # the time to a TRUE relative residual <= tol: a solve that stops on
        # its recurrence residual with the true one above tol (BiCG's
        # recurrence drifts) is repeated with the tolerance tightened by the
        # gap, at most twice; the solve that reached tol is the one timed
        run_tol = tol
        for attempt in range(3):
            psi.zero_()
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            perf = cf._TABLE[solver]("U", M, dict(ctrl, tolerance=run_tol)).solve(psi, src)
            torch.cuda.synchronize()
            wall = time.perf_counter() - w0
            r = src - M.spmv(psi, row_order="fast")
            true_rel = float(torch.linalg.norm(r)) / perf.norm_factor
            if perf.status_name != "ok" or true_rel <= tol or attempt == 2:
                break
            run_tol = run_tol * 0.8 * tol / true_rel
        res[prec] = (psi, perf)
        out[prec] = {"ms": round(perf.solve_ms, 2), "wall_ms": round(1e3 * wall, 2),
                     "iterations": perf.n_iterations, "status": perf.status_name,
                     "final_rel_residual": perf.final_residual, "true_rel_residual": true_rel}
        if run_tol != tol:
            out[prec]["tightened_tolerance"] = run_tol
        if prec == "mixed":
            out[prec]["refinements"] = perf.n_outer
    (x64, p64), (x32, p32) = res["FP64"], res["mixed"]
    out["mixed"]["rel_error_vs_fp64"] = float(torch.linalg.norm(x32 - x64) / torch.linalg.norm(x64))
    def reached(prec):   # converged with the true residual at the target
        return out[prec]["status"] == "ok" and out[prec]["true_rel_residual"] <= tol
    both = reached("FP64") and reached("mixed")
    out["speedup"] = round(p64.solve_ms / p32.solve_ms, 3) if both else None
    if "FP64_fast" in res:
        pf = res["FP64_fast"][1]
        ok = reached("FP64_fast") and reached("mixed")
        out["speedup_vs_fast"] = round(pf.solve_ms / p32.solve_ms, 3) if ok else None
    M.close()
    return out


def batched_vs_sequential(ctx, device, n_systems: int = 512, tol: float = 1e-8,
                          max_iter: int = 5000):
    """512 lognormal 7-point systems (box sides uniform in 16..64, rows
    randomly permuted) x 3 right-hand sides: one persistent batched launch
    vs one cuFoamCG solve per (system, right-hand side)."""
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    from cufoam_gb300.batch import BatchSolver, c4_systems
    t0 = time.perf_counter()
    systems, sizes = c4_systems(n_systems, seed=4)
    rhs = [np.stack([W.uniform(10_000 + 3 * s + j, L.n) for j in range(3)])
           for s, L in enumerate(systems)]
    gen_s = time.perf_counter() - t0
    B = BatchSolver(systems, n_rhs=3, context=ctx)
    dev = f"cuda:{device}"
    packed = torch.from_numpy(B.pack(rhs)).to(dev)
    cands = [(4, 256, 0), (8, 256, 0), (16, 256, 0), (16, 128, 0), (4, 512, 0)]
    cfg, entry = B.tune(packed, tolerance=tol, max_iter=max_iter, candidates=cands, use_cache=False)
    x, res, ms = B.solve(packed, tolerance=tol, max_iter=max_iter)
    torch.cuda.synchronize()
    n_solves = 3 * n_systems
    ok = sum(1 for r in res if r["status"] == 0)
    # the same batch in mixed precision (FP32 CG sweeps, FP64 refinement)
    cfg32, _ = B.tune(packed, tolerance=tol, max_iter=max_iter, candidates=cands, use_cache=False,
                      precision="mixed")
    x32, res32, ms32 = B.solve(packed, tolerance=tol, max_iter=max_iter, precision="mixed")
    torch.cuda.synchronize()
    ok32 = sum(1 for r in res32 if r["status"] == 0)
    err32 = float(torch.linalg.norm(x32 - x) / torch.linalg.norm(x))
    # sequential: one solve per (system, rhs) through the plugin path, device vectors
    mats = [cf.LduMatrix.from_ldu(L, ctx) for L in systems]
    srcs = [[torch.from_numpy(np.ascontiguousarray(rhs[s][j])).to(dev) for j in range(3)]
            for s in range(n_systems)]
    psis = [torch.zeros(L.n, dtype=torch.float64, device=dev) for L in systems]
    solver_ctrl = {"tolerance": tol, "maxIter": max_iter}
    cf.cuFoamCG("U", mats[0], solver_ctrl).solve(psis[0], srcs[0][0])
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream(device)
    e0.record(stream)
    seq_iters = 0
    for s in range(n_systems):
        sol = cf.cuFoamCG("U", mats[s], solver_ctrl)
        for j in range(3):
            psis[s].zero_()
            seq_iters += sol.solve(psis[s], srcs[s][j]).n_iterations
    e1.record(stream)
    torch.cuda.synchronize()
    seq_ms = e0.elapsed_time(e1)
    for m in mats:
        m.close()
    B.close()
    return {"workload": f"{n_systems} lognormal 7-point boxes (16..64)^3 permuted x 3 rhs, CG FP64",
            "rows": int(sizes.prod(axis=1).sum()), "tolerance": tol, "generate_s": round(gen_s, 1),
            "autotuned": {"cluster": cfg[0], "threads": cfg[1], "order": cfg[2]},
            "batched_ms": round(ms, 2), "batched_solves_per_s": round(n_solves / (ms * 1e-3), 1),
            "batched_converged": ok, "sequential_ms": round(seq_ms, 2),
            "sequential_solves_per_s": round(n_solves / (seq_ms * 1e-3), 1),
            "speedup": round(seq_ms / ms, 3),
            "iterations_batched": int(sum(r["n_iterations"] for r in res)),
            "iterations_sequential": int(seq_iters),
            "mixed": {"autotuned": {"cluster": cfg32[0], "threads": cfg32[1], "order": cfg32[2]},
                      "batched_ms": round(ms32, 2),
                      "batched_solves_per_s": round(n_solves / (ms32 * 1e-3), 1),
                      "converged": ok32, "speedup_vs_sequential_fp64": round(seq_ms / ms32, 3),
                      "speedup_vs_batched_fp64": round(ms / ms32, 3),
                      "rel_error_vs_batched_fp64": err32,
                      "iterations": int(sum(r["n_iterations"] for r in res32))}}


def run_profile(args):
    """A short run for ncu: the same 128^3 CG solve with host-driven
    launches (every kernel a separate launch), then five plain SpMVs over the
    one-byte column codes (k_spmv_sell<1>) and five over the 32-bit columns
    (k_spmv_sell<0>)."""
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    L, b = make_problem()
    ctx = cf.Context(0)
    M = cf.LduMatrix.from_ldu(L, ctx)
    src = torch.from_numpy(b).cuda()
    psi = torch.zeros(L.n, dtype=torch.float64, device="cuda")
    s = cf.cuFoamCG("p", M, {"tolerance": TOL, "maxIter": MAX_ITER, "useGraph": 0})
    for _ in range(args.steps):
        psi.zero_()
        perf = s.solve(psi, src)
    x = torch.from_numpy(W.uniform(5, L.n)).cuda()
    for fmt in ("auto", "sell"):
        M.set_format(fmt)
        for _ in range(5):
            M.spmv(x, row_order="fast")
    torch.cuda.synchronize()
    print(f"profile run ok: {perf.n_iterations} iterations")
    return 0


def run_profile_mr(args):
    """A short run for ncu: MR on the 256^3 upwind convection-diffusion
    system, FP64 and mixed precision, 300 steps each, host-driven launches."""
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    ctx = cf.Context(0)
    L, _ = W.grid_convdiff(256, 256, 256, 7, 10.0)
    M = cf.LduMatrix.from_ldu(L, ctx)
    src = torch.from_numpy(W.uniform(8, L.n)).cuda()
    for prec in ("FP64", "mixed"):
        psi = torch.zeros(L.n, dtype=torch.float64, device="cuda")
        perf = cf.cuFoamMR("U", M, {"tolerance": 1e-10, "maxIter": 300, "precision": prec,
                                    "innerMaxIter": 300, "useGraph": 0}).solve(psi, src)
        print(f"profile run ok: MR {prec} {perf.n_iterations} steps")
    return 0


def run_profile_batch(args, small: bool = False):
    """A batched solve small enough for a full ncu capture: 256 lognormal
    7-point boxes with sides uniform in 16..40, rows permuted, 3 right-hand
    sides, CG to 1e-8 in FP64 and in mixed precision, default schedule.
    small: 32 boxes with sides 16..24 and at most 300 steps, short enough
    launches for ncu's ~40 replay passes of the mixed kernel."""
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    from cufoam_gb300.batch import BatchSolver, c4_systems
    ctx = cf.Context(0)
    systems, _ = c4_systems(32, seed=4, lo=16, hi=24) if small else c4_systems(256, seed=4, lo=16, hi=40)
    B = BatchSolver(systems, n_rhs=3, context=ctx)
    rhs = [np.stack([W.uniform(10_000 + 3 * s + j, L.n) for j in range(3)])
           for s, L in enumerate(systems)]
    packed = torch.from_numpy(B.pack(rhs)).to("cuda")
    for prec in ("FP64", "mixed"):
        _, res, ms = B.solve(packed, tolerance=1e-8, max_iter=300 if small else 5000, precision=prec)
        print(f"{prec}: {ms:.2f} ms, {sum(r['n_iterations'] for r in res)} iterations, "
              f"{sum(r['status'] == 0 for r in res)}/{len(res)} converged")
    B.close()
    ctx.close()
    return 0


def run_profile_scaled(args):
    """A short host-driven run on the 128^3 lognormal Poisson system for an
    ncu capture of the scaled-matrix kernels: 6 FP64 Jacobi steps (one pass
    over A D^-1 each) and 6 FP32 MRJacobi steps (MR on A D^-1) of one
    mixed-precision sweep."""
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    torch.cuda.set_device(0)
    ctx = cf.Context(0)
    ctx.set_stream(torch.cuda.current_stream(0))
    L = W.grid_lognormal(128, 128, 128, 2)
    b = torch.from_numpy(W.uniform(3, L.n)).cuda()
    M = cf.LduMatrix.from_ldu(L, ctx)
    for solver, prec in (("cuFoamJacobi", "FP64"), ("cuFoamMRJacobi", "mixed")):
        psi = torch.zeros(L.n, dtype=torch.float64, device="cuda")
        perf = cf._TABLE[solver]("p", M, {"tolerance": 1e-30, "maxIter": 6, "useGraph": 0,
                                          "precision": prec, "innerMaxIter": 6,
                                          "maxRefinements": 1}).solve(psi, b)
        torch.cuda.synchronize()
        print(solver, prec, perf.n_iterations, perf.status_name, flush=True)
    return 0


def run_profile_all(args):
    """A short run for an ncu launch list of every kernel family: on 128^3
    systems, 20 host-driven steps of each solver in both summation orders
    (and in mixed precision for CG, MR, MRJacobi, JMR and BiCG), the plain
    SpMVs, normFactor,
    the device ldu2csr, one adjoint gradient pass and a small batched solve
    (64 systems x 3 right-hand sides, FP64 and mixed)."""
    import torch

    import cufoam_gb300 as cf
    from cufoam_gb300 import workloads as W
    from cufoam_gb300.batch import BatchSolver, c4_systems
    ctx = cf.Context(0)
    dev = "cuda"
    n3 = 128
    sym = W.grid_lognormal(n3, n3, n3, 2)
    asym, _ = W.grid_convdiff(n3, n3, n3, 3, 10.0)
    Ms = cf.LduMatrix.from_ldu(sym, ctx)
    Ma = cf.LduMatrix.from_ldu(asym, ctx)
    b = torch.from_numpy(W.uniform(3, sym.n)).to(dev)
    steps = 20
    for name in ("cuFoamCG", "cuFoamPCG", "cuFoamJacobi", "cuFoamRichardson", "cuFoamMR",
                 "cuFoamMRJacobi", "cuFoamMRS", "cuFoamJMR", "cuFoamBiCG"):
        M = Ma if name == "cuFoamBiCG" else Ms
        orders = ("fast",) if name == "cuFoamPCG" else ("fast", "reference")
        for red in orders:
            psi = torch.zeros(sym.n, dtype=torch.float64, device=dev)
            cf._TABLE[name]("p", M, {"tolerance": 1e-30, "maxIter": steps, "useGraph": 0,
                                     "reduction": red}).solve(psi, b)
        if name in ("cuFoamCG", "cuFoamMR", "cuFoamMRJacobi", "cuFoamJMR", "cuFoamBiCG"):
            psi = torch.zeros(sym.n, dtype=torch.float64, device=dev)
            cf._TABLE[name]("p", M, {"tolerance": 1e-30, "maxIter": steps, "useGraph": 0,
                                     "precision": "mixed", "innerMaxIter": steps,
                                     "maxRefinements": 2}).solve(psi, b)
    x = torch.from_numpy(W.uniform(5, sym.n)).to(dev)
    y = torch.empty_like(x)
    for row_order in ("fast", "reference"):
        Ms.spmv(x, row_order=row_order, out=y)
        Ms.spmv(x, transpose=True, row_order=row_order, out=y)
    for red in ("fast", "reference"):
        Ms.norm_factor(b, x, reduction=red)
    cf.LduMatrix.from_ldu(asym, ctx).close()     # one more device ldu2csr, asymmetric
    lam = torch.from_numpy(W.uniform(7, sym.n)).to(dev)
    dd, dl, du = (torch.empty(k, dtype=torch.float64, device=dev)
                  for k in (sym.n, Ms.n_faces, Ms.n_faces))
    torch.cuda.synchronize()
    ctx.check(Ms._lib.cf_adjoint_gradients(Ms.handle, lam.data_ptr(), x.data_ptr(), dd.data_ptr(),
                                           dl.data_ptr(), du.data_ptr(), 1), "cf_adjoint_gradients")
    systems, _ = c4_systems(64, seed=4)
    B = BatchSolver(systems, n_rhs=3, context=ctx)
    rhs = [np.stack([W.uniform(10_000 + 3 * s + j, L.n) for j in range(3)])
           for s, L in enumerate(systems)]
    packed = torch.from_numpy(B.pack(rhs)).to(dev)
    for prec in ("FP64", "mixed"):
        B.solve(packed, tolerance=1e-8, max_iter=200, config=(4, 256, 0), precision=prec)
    torch.cuda.synchronize()
    print("profile run ok: all kernel families")
    return 0


# Algorithmic bytes per launch of every kernel family in the `--profile-all`
# run (128^3 7-point systems), as (label, bytes) from the sizes: N cells, F
# faces, nnz CSR entries, S stored SELL-32 entries in `slices` slices.  V =
# one FP64 vector, V32 = one FP32 vector; a gathered vector counts once.
def _launch_bytes(N, F, nnz, S, slices):
    V, V32 = 8 * N, 4 * N
    Mcsr = 12 * nnz + 4 * (N + 1)
    Msell = 12 * S + 4 * (slices + 1)
    Msell32 = 8 * S + 4 * (slices + 1)
    Msell8 = 9 * S + 4 * (slices + 1) + 128           # one-byte column codes (format 2)
    Msell8_32 = 5 * S + 4 * (slices + 1) + 128
    Msell16 = 10 * S + 4 * (slices + 1)               # 16-bit column deltas (format 3)
    Msell16_32 = 6 * S + 4 * (slices + 1)
    t = {
        "k_pow_step": ("Mcsr + 2V", Mcsr + 2 * V), "k_pow_final": ("Mcsr + V", Mcsr + V),
        "k_bicg_spmv": ("Mcsr + 8nnz + 10V", Mcsr + 8 * nnz + 10 * V),
        "k_mr_spmv<0>": ("Mcsr + 2V", Mcsr + 2 * V), "k_mr_spmv<1>": ("Mcsr + 3V", Mcsr + 3 * V),
        "k_mr_spmv<2>": ("Mcsr + 3V", Mcsr + 3 * V), "k_mr_spmv<3>": ("Mcsr + 4V", Mcsr + 4 * V),
        "k_nf_dist": ("Mcsr + 2V", Mcsr + 2 * V), "k_nf_sum": ("V", V),
        "k_jacobi_step": ("Mcsr + 5V", Mcsr + 5 * V), "k_rich_step": ("Mcsr + 5V", Mcsr + 5 * V),
        "k_cg_spmv": ("Mcsr + 6V", Mcsr + 6 * V), "k_res_init": ("Mcsr + 3V", Mcsr + 3 * V),
        "k_bicg_update": ("6V", 6 * V), "k_cg_update": ("3V", 3 * V),
        "k_mr_update<0>": ("5V", 5 * V), "k_mr_update<1>": ("6V", 6 * V),
        "k_mr_update<2>": ("6V", 6 * V), "k_mr_update<3>": ("6V", 6 * V),
        "k_f_cg_spmv<1>": ("Msell + 2V", Msell + 2 * V), "k_f_cg_update": ("3V", 3 * V),
        "k_f_cg_prep": ("5V", 5 * V), "k_f_pcg_prep": ("6V", 6 * V), "k_f_pcg_update": ("4V", 4 * V),
        "k_f_bicg_spmv<1>": ("Msell + 8S + 4V", Msell + 8 * S + 4 * V),
        "k_f_bicg_prep": ("8V", 8 * V), "k_f_bicg_update": ("6V", 6 * V),
        "k_f_jac_step<1>": ("Msell + 5V", Msell + 5 * V),
        "k_f_rich_spmv<1>": ("Msell + 3V", Msell + 3 * V), "k_f_rich_prep": ("3V", 3 * V),
        "k_f_mr_spmv<0, 1>": ("Msell + 2V", Msell + 2 * V),
        "k_f_mr_spmv<1, 1>": ("Msell + 2V", Msell + 2 * V),
        "k_f_mr_spmv<2, 1>": ("Msell + 3V", Msell + 3 * V),
        "k_f_mr_update<0>": ("5V", 5 * V), "k_f_mr_update<1>": ("6V", 6 * V),
        "k_f_mr_update<2>": ("8V", 8 * V),
        "k_f_flush_x": ("3V", 3 * V), "k_flush_x": ("3V", 3 * V), "k_rich_finish": ("2V", 2 * V),
        "k_min_abs": ("V", V),
        "k_mx_mr_spmv<1>": ("Msell32 + 2V32", Msell32 + 2 * V32), "k_mx_mr_update": ("5V32", 5 * V32),
        "k_mx_cg_spmv<1>": ("Msell32 + 6V32", Msell32 + 6 * V32), "k_mx_cg_update": ("3V32", 3 * V32),
        "k_mx_bcs_spmv1<1>": ("Msell32 + 3V32", Msell32 + 3 * V32),
        "k_mx_bcs_spmv2<1>": ("Msell32 + 4V32", Msell32 + 4 * V32),
        "k_mx_bcs_prep": ("4V32", 4 * V32), "k_mx_bcs_update": ("7V32", 7 * V32),
        "k_mx_residual<1, 0>": ("Msell + 3V", Msell + 3 * V),
        "k_mx_residual<1, 1>": ("Msell + 4V", Msell + 4 * V),
        "k_mx_setup": ("V + 2V32", V + 2 * V32), "k_mx_correct": ("2V + V32", 2 * V + V32),
        "k_mx_flush": ("3V32", 3 * V32),
        "k_scaled_sell<float>": ("16S + V", 16 * S + V), "k_scaled_sell<double>": ("20S + V", 20 * S + V),
        "k_spmv_sell": ("Msell + 2V", Msell + 2 * V),
        "k_spmv_sell_ref": ("Msell + 4(N+1) + 2V", Msell + 4 * (N + 1) + 2 * V),
        "k_adjoint_faces": ("24F + 2V", 24 * F + 2 * V), "k_adjoint_cells": ("3V", 3 * V),
    }
    # the same passes over the one-byte column codes: format 2 in the kernel
    # name, Msell8 (Msell8_32 for FP32 values) in place of Msell (Msell32)
    # and over the 16-bit deltas: format 3, Msell16 (Msell16_32)
    for name, (formula, val) in list(t.items()):
        if not (name.startswith("k_f_") or name.startswith("k_mx_")) or "Msell" not in formula:
            continue
        for fmt, m64, m32 in ((2, Msell8, Msell8_32), (3, Msell16, Msell16_32)):
            lab = "Msell8" if fmt == 2 else "Msell16"
            if name.startswith("k_mx_residual"):
                n2 = name.replace("<1, ", f"<{fmt}, ")
            elif name.startswith("k_f_mr_spmv"):
                n2 = name.replace(", 1>", f", {fmt}>")
            else:
                n2 = name.replace("<1>", f"<{fmt}>")
            if "Msell32" in formula:
                t[n2] = (formula.replace("Msell32", lab + "_32"), val - Msell32 + m32)
            else:
                t[n2] = (formula.replace("Msell", lab), val - Msell + m64)
    t["k_spmv_sell<1>"] = ("Msell8 + 2V", Msell8 + 2 * V)     # over the one-byte codes
    t["k_spmv_sell<2>"] = ("Msell16 + 2V", Msell16 + 2 * V)   # over the 16-bit deltas
    t["k_spmv_sell<0>"] = t["k_spmv_sell"]
    return t


def launch_table(csv_path: str, N: int = 2_097_152, F: int = 6_242_304, nnz: int = 14_581_760,
                 S: int = 14_614_528, slices: int = 65_536) -> str:
    """The markdown launch table of an ncu `gpu__time_duration.sum` CSV of
    `--profile-all`: per kernel family its launches (working launches: those
    of at least 40% of the family's longest -- host-driven loops launch
    chunks whose steps after convergence return at once), total time,
    share, mean working time, algorithmic bytes per launch and GB/s."""
    import csv
    import collections
    rows = list(csv.reader(open(csv_path)))
    hi = next(i for i, r in enumerate(rows) if r and r[0] == "ID")
    h = rows[hi]
    ki, vi, ui = h.index("Kernel Name"), h.index("Metric Value"), h.index("Metric Unit")
    scale = {"ns": 1e-3, "nsecond": 1e-3, "us": 1.0, "usecond": 1.0, "ms": 1e3, "msecond": 1e3,
             "s": 1e6, "second": 1e6}
    times = collections.defaultdict(list)
    for r in rows[hi + 1:]:
        if len(r) <= vi or not r[vi]:
            continue
        name = r[ki].split("(")[0].replace("void ", "").replace("cf::", "").strip()
        times[name].append(float(r[vi].replace(",", "")) * scale.get(r[ui], 1.0))
    table = _launch_bytes(N, F, nnz, S, slices)
    total = sum(sum(v) for v in times.values())
    out = ["| kernel | launches (working) | total ms | share | mean µs (working) | "
           "algorithmic bytes / launch | GB/s |", "|---|---|---|---|---|---|---|"]
    for name, ts in sorted(times.items(), key=lambda kv: -sum(kv[1])):
        work = [t for t in ts if t >= 0.4 * max(ts)]
        mean = sum(work) / len(work)
        label, nbytes = table.get(name, ("set-up / persistent (see note)", None))
        gbs = f"{nbytes / (mean * 1e-6) / 1e9:,.0f}" if nbytes else "—"
        lab = f"{label} = {nbytes / 1e6:.1f} MB" if nbytes else label
        out.append(f"| `{name}` | {len(ts)} ({len(work)}) | {sum(ts) / 1e3:.3f} | "
                   f"{100 * sum(ts) / total:.1f}% | {mean:,.2f} | {lab} | {gbs} |")
    out.append(f"\n{len(times)} kernels, {total / 1e3:.1f} ms in total")
    return "\n".join(out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the mixed-vs-FP64 and batched-vs-sequential comparisons")
    ap.add_argument("--profile", action="store_true",
                    help="short host-driven run for an ncu capture (prints no JSON)")
    ap.add_argument("--profile-batch-small", action="store_true",
                    help="the same with 32 systems of sides 16..24 and at most 300 steps (ncu --set full)")
    ap.add_argument("--profile-batch", action="store_true",
                    help="one FP64 and one mixed batched solve of 256 small systems, for ncu")
    ap.add_argument("--profile-all", action="store_true",
                    help="short run launching every kernel family once, for an ncu launch list")
    ap.add_argument("--profile-mr", action="store_true",
                    help="short host-driven MR run (FP64 and mixed, 256^3) for an ncu capture")
    ap.add_argument("--launch-table", metavar="CSV",
                    help="print the markdown launch table of an ncu CSV of --profile-all")
    ap.add_argument("--launch-sizes", metavar="N,F,NNZ,S,SLICES",
                    help="system sizes for --launch-table (default: the 128^3 7-point system)")
    ap.add_argument("--profile-scaled", action="store_true",
                    help="6 Jacobi (FP64) and 6 mixed MRJacobi steps at 128^3, for an ncu capture")
    args = ap.parse_args()
    if args.profile_scaled:
        return run_profile_scaled(args)
    if args.launch_table:
        sizes = [int(v) for v in args.launch_sizes.split(",")] if args.launch_sizes else []
        print(launch_table(args.launch_table, *sizes))
        return 0
    if args.profile_mr:
        return run_profile_mr(args)
    if args.profile_all:
        return run_profile_all(args)
    if args.profile_batch or args.profile_batch_small:
        return run_profile_batch(args, small=args.profile_batch_small)
    if args.profile:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
