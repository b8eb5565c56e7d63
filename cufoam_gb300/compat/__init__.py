"""libGIS.so compatibility: ``_build/libGIS.so`` exports the reference solver
library's gis.h functions (CG, BiCG, Richardson, MR, Jacobi, MRJacobi, JMR,
MRS, NormFactor, Transpose) on this library's device solvers, so the
unmodified cuFoam plugins can link against it.  ``GisHarness`` drives it
through ``_build/libgis_harness.so`` the way the plugins do (device
containers built with cudaMalloc, one solver call) from host arrays."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ..build import GIS_HARNESS, GIS_LIB, build_gis  # noqa: F401

_P = C.c_void_p


class GisError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code   # 1 runtime_error, 2 invalid_argument


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class GisHarness:
    SOLVERS = ("CG", "BiCG", "BiCGAt", "Richardson", "MR", "Jacobi", "MRJacobi", "JMR", "MRS")

    def __init__(self, path: str = GIS_HARNESS):
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} not built (cufoam_gb300.build.build_gis)")
        self.lib = C.CDLL(path)
        L = self.lib
        L.gh_last_error.restype = C.c_char_p
        L.gh_layout.argtypes = [C.POINTER(C.c_long)]
        L.gh_solve.restype = C.c_int
        L.gh_solve.argtypes = [C.c_char_p, C.c_int, C.c_int, _P, _P, _P, C.c_int, _P, C.c_int, _P,
                               C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, _P, C.c_int,
                               C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.gh_transpose.restype = C.c_int
        L.gh_transpose.argtypes = [C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P]
        L.gh_norm_factor.restype = C.c_int
        L.gh_norm_factor.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, _P, C.POINTER(C.c_double)]

    def _check(self, rc: int):
        if rc != 0:
            raise GisError(rc, self.lib.gh_last_error().decode())

    def layout(self) -> list[int]:
        a = (C.c_long * 9)()
        self.lib.gh_layout(a)
        return list(a)

    def solve(self, name: str, ro, cols, vals, b, x0, error: float, max_steps: int,
              p_real: float = 0.0, p_int: int = 30, detail: str | None = "error",
              detail_cap: int | None = None):
        """Returns (x, detail list, BiCG's return value)."""
        ro, cols, vals, b = _i32(ro), _i32(cols), _f64(vals), _f64(b)
        x = _f64(np.array(x0, dtype=np.float64, copy=True))
        n = ro.shape[0] - 1
        cap = detail_cap if detail_cap is not None else (max_steps + 1 if max_steps > 0 else 1 << 16)
        det = np.zeros(max(cap, 1))
        dl, flag = C.c_int(0), C.c_int(0)
        dt = {None: -1, "error": 0, "time": 1}[detail]
        self._check(self.lib.gh_solve(name.encode(), n, vals.shape[0], ro.ctypes.data, cols.ctypes.data,
                                      vals.ctypes.data, b.shape[0], b.ctypes.data, x.shape[0],
                                      x.ctypes.data, error, max_steps, p_real, p_int, dt,
                                      det.ctypes.data, cap, C.byref(dl), C.byref(flag)))
        return x, det[:min(dl.value, cap)].copy(), bool(flag.value)

    def transpose(self, n_rows: int, n_cols: int, ro, cols, vals):
        ro, cols, vals = _i32(ro), _i32(cols), _f64(vals)
        nnz = vals.shape[0]
        roT = np.zeros(n_cols + 1, np.int32)
        colT = np.zeros(max(nnz, 1), np.int32)
        valT = np.zeros(max(nnz, 1))
        shape = (C.c_int * 3)()
        self._check(self.lib.gh_transpose(n_rows, n_cols, nnz, ro.ctypes.data, cols.ctypes.data,
                                          vals.ctypes.data, roT.ctypes.data, colT.ctypes.data,
                                          valT.ctypes.data, shape))
        return tuple(shape), roT, colT[:nnz], valT[:nnz]

    def norm_factor(self, ro, cols, vals, b, x) -> float:
        ro, cols, vals, b, x = _i32(ro), _i32(cols), _f64(vals), _f64(b), _f64(x)
        out = C.c_double()
        self._check(self.lib.gh_norm_factor(ro.shape[0] - 1, vals.shape[0], ro.ctypes.data,
                                            cols.ctypes.data, vals.ctypes.data, b.ctypes.data,
                                            x.ctypes.data, C.byref(out)))
        return out.value
