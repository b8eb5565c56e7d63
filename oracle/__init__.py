"""CPU oracle for the cuFoam sparse solve path -- TEST INFRASTRUCTURE ONLY.

(The seeded input generators it re-exports live in cufoam_gb300.workloads;
they make inputs, they do not check anything.)

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this package, and only as the checker / the timed CPU
baseline; the product library never imports it.

It wraps ``oracle.c`` (a plain-C restatement of the reference algorithms,
see ``oracle.h``) with numpy helpers, and exposes the reference's own
``gis/ldu2csr.h`` compiled from source (``oracle/_ref``) where available.

Parity status: ldu2csr pinned to the reference's own code; the solver
restatement's arithmetic is pinned on the GPU by running the same drivers
through the reference's own kernels (``reference_kernels()``, used by
``tests/test_gpu_refgpu.py``); it is also cross-checked against direct
solves.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from cufoam_gb300.workloads import (LDU, diffusion_from_cells, grid_addressing,  # noqa: F401
                                    grid_const, grid_convdiff, grid_grf, grid_lognormal,
                                    n_faces, normal, permutation, permute_ldu, uniform)

from . import build as _build

# solver kinds (same numbering as the C ABI's cf_solver_kind)
CG, BICG, JACOBI, MR, MRJACOBI, MRS, JMR, RICHARDSON = range(8)
SOLVER_NAMES = {"CG": CG, "BiCG": BICG, "Jacobi": JACOBI, "MR": MR,
                "MRJacobi": MRJACOBI, "MRS": MRS, "JMR": JMR,
                "Richardson": RICHARDSON}

# The reference's LaunchConfig grid on a GB300: maxThreadsPerSM (2048) / 256
# threads per block * 152 SMs (gis/SparseSystem/launch.h:116-139).
GB300_REF_GRID = 2048 // 256 * 152

_lib = None
_ref = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class _Csr(C.Structure):
    _fields_ = [("n", C.c_int32), ("nnz", C.c_int32), ("row_offsets", C.c_void_p),
                ("cols", C.c_void_p), ("vals", C.c_void_p)]


class _Res(C.Structure):
    _fields_ = [("n_hist", C.c_int32), ("breakdown", C.c_int32), ("omega", C.c_double),
                ("lambda_max", C.c_double), ("diag_abs_min", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.orc_ldu_addressing.restype = C.c_int32
        L.orc_ldu_addressing.argtypes = [C.c_int32, C.c_int32, _ip, _ip, _ip, _ip, _ip]
        L.orc_ldu2csr.argtypes = [C.c_int32, C.c_int32, _dp, _dp, _dp, _ip, _ip, _ip, _ip, _ip,
                                  _ip, _ip, _dp]
        L.orc_set_threads.argtypes = [C.c_int32]
        L.orc_get_threads.restype = C.c_int32
        for fn in ("orc_ref_dot", "orc_ref_distance"):
            getattr(L, fn).restype = C.c_double
            getattr(L, fn).argtypes = [_dp, _dp, C.c_int32, C.c_int32]
        L.orc_ref_sum.restype = C.c_double
        L.orc_ref_sum.argtypes = [_dp, C.c_int32, C.c_int32]
        L.orc_ref_spmv.argtypes = [C.POINTER(_Csr), _dp, _dp]
        L.orc_ref_residual.argtypes = [C.POINTER(_Csr), _dp, _dp, _dp]
        L.orc_true_residual_norm.restype = C.c_double
        L.orc_true_residual_norm.argtypes = [C.POINTER(_Csr), _dp, _dp]
        L.orc_norm_factor.restype = C.c_double
        L.orc_norm_factor.argtypes = [C.POINTER(_Csr), _dp, _dp, C.c_int32]
        L.orc_set_backend.argtypes = [C.c_void_p]
        L.orc_solve.restype = C.c_int32
        L.orc_solve.argtypes = [C.c_int32, C.POINTER(_Csr), C.POINTER(_Csr), _dp, _dp,
                                C.c_double, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                C.c_int32, _dp, C.c_int32, C.POINTER(_Res)]
        _lib = L
    return _lib


class reference_kernels:
    """Within this context the oracle's drivers run on the reference's own
    device kernels (gis/SparseSystem/kernels.h compiled into
    oracle/_ref/ref_kernels.cubin) launched on `device`, instead of on the
    CPU emulation of their arithmetic.  Needs a GPU and the cubin."""

    def __init__(self, device: int = 0):
        self.device = device
        self._g = None

    @staticmethod
    def available() -> bool:
        return os.path.exists(_build.REF_CUBIN) and os.path.exists(_build.REF_CUBIN_NAMES)

    def __enter__(self):
        g = C.CDLL(_build.build_refgpu())
        g.rg_open.restype = C.c_int
        g.rg_open.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int]
        g.rg_backend.restype = C.c_void_p
        g.rg_grid.restype = C.c_int
        g.rg_launches.restype = C.c_long
        g.rg_error.restype = C.c_int
        g.rg_error.argtypes = [C.c_char_p, C.c_int]
        err = C.create_string_buffer(256)
        if g.rg_open(_build.REF_CUBIN.encode(), _build.REF_CUBIN_NAMES.encode(), self.device, err, 256):
            raise RuntimeError("reference kernels unavailable: " + err.value.decode())
        self._g = g
        self.grid = int(g.rg_grid())
        lib().orc_set_backend(g.rg_backend())
        return self

    def cg_device(self, A, b, x0, error: float, max_steps: int):
        """The reference's CG with its own kernels on device-resident data:
        (x, history, steps, wall ms of the solver call)."""
        g = self._g
        g.rg_cg_device.restype = C.c_int
        g.rg_cg_device.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_double, C.c_int, _dp,
                                   C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        x = np.array(x0, dtype=np.float64, copy=True)
        cap = (max_steps if max_steps > 0 else 100_000) + 1
        hist = np.zeros(cap)
        nh, ms = C.c_int(0), C.c_double(0.0)
        k = g.rg_cg_device(A.n, A.nnz, A.row_offsets, A.cols, A.vals, _f64(b), x, error, max_steps, hist,
                           cap, C.byref(nh), C.byref(ms))
        self.check()
        if k < 0:
            raise RuntimeError("reference CG failed")
        return x, hist[:nh.value].copy(), int(k), float(ms.value)

    def launches(self) -> int:
        """Reference kernels launched since the context opened."""
        return int(self._g.rg_launches())

    def check(self) -> None:
        """Raise if any driver call failed since the context opened."""
        where = C.create_string_buffer(128)
        e = self._g.rg_error(where, 128)
        if e:
            raise RuntimeError(f"CUDA driver error {e} in {where.value.decode()}")

    def __exit__(self, *exc):
        lib().orc_set_backend(None)
        if self._g is not None:
            self._g.rg_close()
            self._g = None
        return False


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


# --------------------------------------------------------------------------
# containers
# --------------------------------------------------------------------------
@dataclass
class CSR:
    row_offsets: np.ndarray
    cols: np.ndarray
    vals: np.ndarray

    @property
    def n(self) -> int:
        return int(self.row_offsets.shape[0] - 1)

    @property
    def nnz(self) -> int:
        return int(self.vals.shape[0])

    def c(self) -> _Csr:
        s = _Csr(self.n, self.nnz, self.row_offsets.ctypes.data, self.cols.ctypes.data,
                 self.vals.ctypes.data)
        s._keep = (self.row_offsets, self.cols, self.vals)
        return s

    def dense(self) -> np.ndarray:
        A = np.zeros((self.n, self.n))
        for i in range(self.n):
            for j in range(self.row_offsets[i], self.row_offsets[i + 1]):
                A[i, self.cols[j]] += self.vals[j]
        return A


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# --------------------------------------------------------------------------
# addressing / ldu2csr
# --------------------------------------------------------------------------
def ldu_addressing(n: int, lower_addr: np.ndarray, upper_addr: np.ndarray):
    la = _i32(lower_addr)
    ua = _i32(upper_addr)
    f = la.shape[0]
    losort = np.empty(f, np.int32)
    lstart = np.empty(n + 1, np.int32)
    ostart = np.empty(n + 1, np.int32)
    rc = lib().orc_ldu_addressing(n, f, la, ua, losort, lstart, ostart)
    if rc != 0:
        raise ValueError("invalid LDU addressing (faces must be sorted by owner, owner < neighbour)")
    return losort, lstart, ostart


def ldu2csr(ldu: LDU) -> CSR:
    losort, lstart, ostart = ldu.addressing() if ldu._addr is not None else \
        ldu_addressing(ldu.n, ldu.lower_addr, ldu.upper_addr)
    n, f = ldu.n, ldu.n_faces
    ro = np.empty(n + 1, np.int32)
    cols = np.empty(n + 2 * f, np.int32)
    vals = np.empty(n + 2 * f, np.float64)
    lib().orc_ldu2csr(n, f, _f64(ldu.diag), _f64(ldu.lower), _f64(ldu.upper),
                      _i32(ldu.lower_addr), _i32(ldu.upper_addr), losort, lstart, ostart,
                      ro, cols, vals)
    return CSR(ro, cols, vals)


def ref_ldu2csr_available() -> bool:
    return _build.build_ref_ldu2csr() is not None


def ref_ldu2csr(ldu: LDU) -> CSR:
    """The reference's own getSparseCSRMat (gis/ldu2csr.h:7-40), compiled from
    its source into oracle/_ref.  Raises if the reference is not mounted."""
    global _ref
    if _ref is None:
        path = _build.build_ref_ldu2csr()
        if path is None:
            raise RuntimeError("reference sources not available to build oracle/_ref")
        R = C.CDLL(path)
        R.ref_ldu2csr.restype = C.c_int
        R.ref_ldu2csr.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _ip, _ip, _ip, _ip, _ip,
                                  _ip, _ip, _dp]
        _ref = R
    losort, lstart, ostart = ldu.addressing() if ldu._addr is not None else \
        ldu_addressing(ldu.n, ldu.lower_addr, ldu.upper_addr)
    n, f = ldu.n, ldu.n_faces
    ro = np.empty(n + 1, np.int32)
    cols = np.empty(n + 2 * f, np.int32)
    vals = np.empty(n + 2 * f, np.float64)
    rc = _ref.ref_ldu2csr(n, f, _f64(ldu.diag), _f64(ldu.lower), _f64(ldu.upper),
                          _i32(ldu.lower_addr), _i32(ldu.upper_addr), losort, lstart, ostart,
                          ro, cols, vals)
    if rc != 0:
        raise RuntimeError("reference ldu2csr failed")
    return CSR(ro, cols, vals)


# --------------------------------------------------------------------------
# reference-order primitives and solvers
# --------------------------------------------------------------------------
def ref_dot(a, b, grid: int = GB300_REF_GRID) -> float:
    a, b = _f64(a), _f64(b)
    return float(lib().orc_ref_dot(a, b, a.shape[0], grid))


def ref_sum(a, grid: int = GB300_REF_GRID) -> float:
    a = _f64(a)
    return float(lib().orc_ref_sum(a, a.shape[0], grid))


def ref_spmv(A: CSR, x) -> np.ndarray:
    y = np.empty(A.n)
    c = A.c()
    lib().orc_ref_spmv(C.byref(c), _f64(x), y)
    return y


def ref_residual(A: CSR, b, x) -> np.ndarray:
    r = np.empty(A.n)
    c = A.c()
    lib().orc_ref_residual(C.byref(c), _f64(b), _f64(x), r)
    return r


def true_residual_norm(A: CSR, b, x) -> float:
    c = A.c()
    return float(lib().orc_true_residual_norm(C.byref(c), _f64(b), _f64(x)))


def norm_factor(A: CSR, b, x, grid: int = GB300_REF_GRID) -> float:
    """NormFactor of gis/gis.cu:106-123 (the L2 variant)."""
    c = A.c()
    return float(lib().orc_norm_factor(C.byref(c), _f64(b), _f64(x), grid))


@dataclass
class SolveResult:
    x: np.ndarray
    history: np.ndarray      # absolute ||r||_2 per recorded step (initial first)
    n_iterations: int
    breakdown: bool = False
    omega: float = 0.0
    lambda_max: float = 0.0
    diag_abs_min: float = 0.0


def solve(kind: int, A: CSR, b, x0, error: float, max_steps: int,
          grid: int = GB300_REF_GRID, At: CSR | None = None, int_bound: float = 1e-10,
          omega: float = 0.0, power_max_steps: int = 30,
          hist_cap: int | None = None) -> SolveResult:
    """Run one of the reference drivers (SolverSingleGPU.h) with absolute
    stopping threshold ``error``."""
    x = _f64(np.array(x0, dtype=np.float64, copy=True))
    if hist_cap is None:
        hist_cap = (max_steps if max_steps > 0 else 1_000_000) + 1
    hist = np.zeros(hist_cap)
    res = _Res()
    ca = A.c()
    cat = At.c() if At is not None else None
    rc = lib().orc_solve(kind, C.byref(ca), C.byref(cat) if cat is not None else None,
                         _f64(b), x, error, max_steps, grid, int_bound, omega,
                         power_max_steps, hist, hist_cap, C.byref(res))
    if rc != 0:
        raise ValueError("oracle solve failed (bad kind or missing transpose)")
    h = hist[:res.n_hist].copy()
    return SolveResult(x, h, max(res.n_hist - 1, 0), bool(res.breakdown), res.omega,
                       res.lambda_max, res.diag_abs_min)


@dataclass
class PluginResult:
    psi: np.ndarray
    norm_factor: float
    initial_residual: float   # normalised by norm_factor
    final_residual: float
    n_iterations: int
    history: np.ndarray       # absolute
    solve: SolveResult


def plugin_solve(kind: int, ldu: LDU, source, psi, tolerance: float, max_iter: int,
                 grid: int = GB300_REF_GRID, hist_cap: int | None = None) -> PluginResult:
    """What a cuFoam<X>::solve call computes (e.g. cuFoamCG/cuFoamCG.C:38-90):
    ldu2csr, NormFactor, the solver at tolerance*normFactor, and the
    solverPerformance fields (here normalised by normFactor)."""
    A = ldu2csr(ldu)
    At = ldu2csr(ldu.transposed()) if kind == BICG else None
    nf = norm_factor(A, source, psi, grid)
    r = solve(kind, A, source, psi, tolerance * nf, max_iter, grid, At=At, hist_cap=hist_cap)
    h = r.history
    return PluginResult(r.x, nf, float(h[0] / nf), float(h[-1] / nf), r.n_iterations, h, r)
