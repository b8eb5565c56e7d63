"""Batched solves: many LDU systems, each with several right-hand sides
(Ux/Uy/Uz sharing one matrix), in one persistent cluster launch, with an
autotuner for the cluster / block schedule.

    batch = BatchSolver([ldu_0, ldu_1, ...], n_rhs=3)
    x, results = batch.solve(sources, tolerance=1e-8, max_iter=5000)

``sources`` is a list (one per system) of arrays shaped [n_rhs][n] or a
single [total_rows][n_rhs] array in the batch layout.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import time

import numpy as np

from . import _capi, default_context


class cf_batch_config(C.Structure):
    _fields_ = [("cluster_size", C.c_int32), ("threads", C.c_int32), ("order", C.c_int32),
                ("max_clusters", C.c_int32), ("reserved", C.c_int32 * 4)]


class cf_batch_result(C.Structure):
    _fields_ = [("initial_residual", C.c_double), ("final_residual", C.c_double),
                ("norm_factor", C.c_double), ("n_iterations", C.c_int32), ("status", C.c_int32)]


def _bind(lib):
    P = C.c_void_p
    lib.cf_batch_create.restype = C.c_int32
    lib.cf_batch_create.argtypes = [P, C.c_int32, C.POINTER(_capi.cf_ldu_view), C.POINTER(P)]
    lib.cf_batch_destroy.restype = None
    lib.cf_batch_destroy.argtypes = [P]
    lib.cf_batch_shape.restype = C.c_int32
    lib.cf_batch_shape.argtypes = [P, C.POINTER(C.c_int32), C.POINTER(C.c_int64), P]
    lib.cf_batch_solve.restype = C.c_int32
    lib.cf_batch_solve.argtypes = [P, C.c_int32, C.POINTER(_capi.cf_controls),
                                   C.POINTER(cf_batch_config), C.c_int32, P, P,
                                   C.POINTER(cf_batch_result), C.POINTER(C.c_double)]
    return lib


# schedule candidates of the autotuner: (cluster size, threads per CTA, order)
CANDIDATES = [(cs, bt, 0) for cs in (1, 2, 4, 8, 16) for bt in (128, 256, 512)] + [(4, 256, 1)]


def _cache_path() -> str:
    return os.environ.get("CUFOAM_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "cufoam_gb300",
                                       "batch_autotune.json"))


class BatchSolver:
    def __init__(self, systems, n_rhs: int = 3, context=None):
        self.ctx = context or default_context()
        self._lib = _bind(self.ctx._lib)
        self.n_rhs = int(n_rhs)
        self.systems = list(systems)
        views = (_capi.cf_ldu_view * len(self.systems))()
        keep = []
        for i, L in enumerate(self.systems):
            arrs = [np.ascontiguousarray(L.diag, np.float64), np.ascontiguousarray(L.lower, np.float64),
                    np.ascontiguousarray(L.upper, np.float64), np.ascontiguousarray(L.lower_addr, np.int32),
                    np.ascontiguousarray(L.upper_addr, np.int32)]
            keep.append(arrs)
            views[i] = _capi.cf_ldu_view(n_cells=L.n, n_faces=arrs[1].shape[0], diag=arrs[0].ctypes.data,
                                         lower=arrs[1].ctypes.data, upper=arrs[2].ctypes.data,
                                         lower_addr=arrs[3].ctypes.data, upper_addr=arrs[4].ctypes.data,
                                         memory=0)
        h = C.c_void_p()
        self.ctx.check(self._lib.cf_batch_create(self.ctx.handle, len(self.systems), views, C.byref(h)),
                       "cf_batch_create")
        self._h = h
        ns, rows = C.c_int32(), C.c_int64()
        offs = np.zeros(len(self.systems), np.int64)
        self._lib.cf_batch_shape(h, C.byref(ns), C.byref(rows), offs.ctypes.data)
        self.rows = rows.value
        self.offsets = offs
        self.sizes = np.array([L.n for L in self.systems], np.int64)
        self.config = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- layout helpers ---------------------------------------------------
    def pack(self, per_system) -> np.ndarray:
        """[n_rhs][n] arrays per system -> the batch layout [rows][n_rhs]."""
        out = np.empty((self.rows, self.n_rhs))
        for s, arr in enumerate(per_system):
            a = np.asarray(arr, np.float64).reshape(self.n_rhs, -1)
            out[self.offsets[s]:self.offsets[s] + a.shape[1]] = a.T
        return out

    def unpack(self, packed) -> list:
        packed = np.asarray(packed).reshape(self.rows, self.n_rhs)
        return [packed[self.offsets[s]:self.offsets[s] + self.sizes[s]].T.copy()
                for s in range(len(self.systems))]

    # ---- solve ------------------------------------------------------------
    def solve(self, sources, psi=None, tolerance: float = 1e-6, max_iter: int = 1000,
              config=None, use_graph: bool = True, precision: str = "FP64",
              inner_rtol: float = 1e-6):
        """Returns (psi in the batch layout, per-(system, rhs) results, device ms).
        precision "mixed": FP32 CG sweeps (inner relative tolerance
        `inner_rtol`) inside FP64 refinement; n_iterations counts FP32 steps.
        The inner tolerance's default 1e-6 measured fastest on the
        512-system Poisson batch at 1e-8 (1.39 s, against 1.47 s at 1e-4 and
        1.41 s at 1e-7: fewer refinement sweeps)."""
        if isinstance(sources, (list, tuple)):
            sources = self.pack(sources)
        if _is_torch(sources):
            mem = _capi.CF_MEM_DEVICE
            b = sources
            x = psi if psi is not None else b.new_zeros(b.shape)
            pb, px = b.data_ptr(), x.data_ptr()
        else:
            mem = _capi.CF_MEM_HOST
            b = np.ascontiguousarray(sources, np.float64).reshape(self.rows, self.n_rhs)
            x = np.zeros_like(b) if psi is None else psi
            pb, px = b.ctypes.data, x.ctypes.data
        c = _capi.cf_controls()
        self._lib.cf_controls_init(C.byref(c))
        c.tolerance = tolerance
        c.max_iter = max_iter
        c.memory = mem
        c.use_graph = 1 if use_graph else 0
        c.precision = {"FP64": _capi.CF_PREC_FP64, "mixed": _capi.CF_PREC_MIXED}[precision]
        c.mixed_inner_rtol = inner_rtol
        cfg = cf_batch_config()
        cs, bt, order = config or self.config or (0, 256, 0)   # cluster 0: the library picks 16 or 8
        cfg.cluster_size, cfg.threads, cfg.order = cs, bt, order
        res = (cf_batch_result * (len(self.systems) * self.n_rhs))()
        ms = C.c_double()
        if mem == _capi.CF_MEM_DEVICE:
            import torch
            self.ctx.set_stream(torch.cuda.current_stream(b.device))
        self.ctx.check(self._lib.cf_batch_solve(self._h, _capi.CF_CG, C.byref(c), C.byref(cfg),
                                                self.n_rhs, pb, px, res, C.byref(ms)),
                       "cf_batch_solve")
        out = [{"initial_residual": r.initial_residual, "final_residual": r.final_residual,
                "norm_factor": r.norm_factor, "n_iterations": r.n_iterations, "status": r.status}
               for r in res]
        return x, out, ms.value

    # ---- autotuner ---------------------------------------------------------
    def signature(self) -> str:
        hist = np.histogram(np.log2(self.sizes), bins=12, range=(8, 26))[0]
        info = self.ctx.device_info()
        key = f"{info['name']}|{self.n_rhs}|{len(self.systems)}|{hist.tolist()}"
        return hashlib.sha1(key.encode()).hexdigest()[:16]

    def tune(self, sources, tolerance: float = 1e-6, max_iter: int = 1000, reps: int = 1,
             candidates=None, use_cache: bool = True, verbose: bool = False,
             precision: str = "FP64"):
        """Time every schedule candidate on this batch, keep the fastest and
        remember it per (device, size histogram) in a JSON cache."""
        path = _cache_path()
        sig = self.signature() + ("" if precision == "FP64" else "|" + precision)
        cache = {}
        if use_cache and os.path.exists(path):
            try:
                cache = json.load(open(path))
            except Exception:
                cache = {}
            if sig in cache:
                self.config = tuple(cache[sig]["config"])
                return self.config, cache[sig]
        timings = {}
        for cand in candidates or CANDIDATES:
            best = None
            for _ in range(reps):
                _, out, ms = self.solve(sources, tolerance=tolerance, max_iter=max_iter, config=cand,
                                        precision=precision)
                best = ms if best is None else min(best, ms)
            timings[cand] = best
            if verbose:
                print(f"  cluster={cand[0]} threads={cand[1]} order={cand[2]}: {best:.3f} ms")
        self.config = min(timings, key=timings.get)
        entry = {"config": list(self.config),
                 "timings_ms": {f"{k[0]}x{k[1]}/{k[2]}": v for k, v in timings.items()},
                 "when": time.time()}
        if use_cache:
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                cache[sig] = entry
                with open(path + ".tmp", "w") as f:
                    json.dump(cache, f, indent=1)
                os.replace(path + ".tmp", path)
            except OSError:
                pass
        return self.config, entry


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def c4_systems(n_systems: int = 512, seed: int = 4, lo: int = 16, hi: int = 64):
    """The batch workload: n_systems 7-point systems with lognormal(0,1)
    face coefficients, box sizes nx, ny, nz each uniform in {lo..hi}, rows
    symmetrically permuted at random (P A P^T)."""
    from . import workloads as W
    u = W.uniform(seed, 3 * n_systems, 0.0, 1.0)
    sizes = (lo + np.floor(u * (hi - lo + 1))).astype(int).clip(lo, hi).reshape(n_systems, 3)
    systems = []
    for s in range(n_systems):
        nx, ny, nz = (int(v) for v in sizes[s])
        L = W.grid_lognormal(nx, ny, nz, 1000 + s)
        perm = W.permutation(5000 + s, L.n)
        systems.append(W.permute_ldu(L, perm))
    return systems, sizes
