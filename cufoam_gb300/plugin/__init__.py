"""Access to the C++ plugin layer (cuFoamGB300.{H,C}) compiled against the
minifoam stand-in: ``foam_solve`` runs a plugin exactly as OpenFOAM would
(lduMatrix::solver::New by name, then solve(psi, source, cmpt))."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .. import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _build.build()
        from .. import _capi
        _capi.load()  # the plugin library links against it
        L = C.CDLL(_build.PLUGIN_LIB)
        L.mf_solve.restype = C.c_int
        L.mf_solve.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                               C.c_double, C.c_int, C.c_int, C.POINTER(C.c_char_p),
                               C.POINTER(C.c_char_p), C.c_void_p, C.c_char_p, C.c_int]
        L.mf_solve_coupled.restype = C.c_int
        L.mf_solve_coupled.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_double, C.c_double, C.c_int, C.c_int,
                                       C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_char_p, C.c_int]
        L.mf_solve_reused_addressing.restype = C.c_int
        L.mf_solve_reused_addressing.argtypes = [C.c_int] + list(L.mf_solve.argtypes)
        L.cuFoamGB300_matrix_builds.restype = C.c_long
        L.cuFoamGB300_matrix_builds.argtypes = []
        _lib = L
    return _lib


def matrix_builds() -> int:
    """Device matrices the plugin has built so far (its cache misses)."""
    return int(lib().cuFoamGB300_matrix_builds())


class FoamError(RuntimeError):
    pass


def foam_solve(solver: str, ldu, source, psi, tolerance: float = 1e-6, rel_tol: float = 0.0,
               max_iter: int = 1000, symmetric: bool | None = None, cyclic=None,
               processor_patch: bool = False, reuse_addressing: int | None = None, **controls):
    """Run the plugin `solver` on an LDU matrix through the OpenFOAM-style
    interface; psi (float64 array) is updated in place.  Returns the
    solverPerformance fields as a dict.  cyclic = (faceCellsA, faceCellsB,
    coeffsA, coeffsB) adds a cyclic patch pair (interfaceBouCoeffs coeffs);
    processor_patch adds a processor interface; reuse_addressing = slot
    (0..3) builds the mesh in the memory of the previous mesh of that slot
    (same addressing object and list buffers), as a running case keeps its
    meshes."""
    if symmetric is None:
        symmetric = np.array_equal(ldu.lower, ldu.upper)
    d = np.ascontiguousarray(ldu.diag, np.float64)
    lo = np.ascontiguousarray(ldu.lower, np.float64)
    up = np.ascontiguousarray(ldu.upper, np.float64)
    la = np.ascontiguousarray(ldu.lower_addr, np.int32)
    ua = np.ascontiguousarray(ldu.upper_addr, np.int32)
    b = np.ascontiguousarray(source, np.float64)
    if psi.dtype != np.float64 or not psi.flags["C_CONTIGUOUS"]:
        raise TypeError("psi must be a contiguous float64 array")
    keys = [k.encode() for k in controls]
    vals = [str(v).encode() for v in controls.values()]
    ck = (C.c_char_p * max(1, len(keys)))(*keys)
    cv = (C.c_char_p * max(1, len(vals)))(*vals)
    out = np.zeros(4)
    err = C.create_string_buffer(1024)
    if cyclic is None and not processor_patch:
        fn = lib().mf_solve if reuse_addressing is None else \
            (lambda *a: lib().mf_solve_reused_addressing(int(reuse_addressing), *a))
        rc = fn(solver.encode(), ldu.n, lo.shape[0], d.ctypes.data,
                            None if symmetric else lo.ctypes.data, up.ctypes.data, la.ctypes.data,
                            ua.ctypes.data, b.ctypes.data, psi.ctypes.data, tolerance, rel_tol,
                            max_iter, len(keys), ck, cv, out.ctypes.data, err, 1024)
    else:
        fa, fb, ca, cb = cyclic if cyclic is not None else ([], [], [], [])
        fa, fb = np.ascontiguousarray(fa, np.int32), np.ascontiguousarray(fb, np.int32)
        ca, cb = np.ascontiguousarray(ca, np.float64), np.ascontiguousarray(cb, np.float64)
        if not (fa.shape == fb.shape == ca.shape == cb.shape):
            raise ValueError("cyclic patch arrays must have one length")
        rc = lib().mf_solve_coupled(solver.encode(), ldu.n, lo.shape[0], d.ctypes.data,
                                    None if symmetric else lo.ctypes.data, up.ctypes.data,
                                    la.ctypes.data, ua.ctypes.data, b.ctypes.data, psi.ctypes.data,
                                    tolerance, rel_tol, max_iter, len(keys), ck, cv, int(fa.shape[0]),
                                    fa.ctypes.data, fb.ctypes.data, ca.ctypes.data, cb.ctypes.data,
                                    1 if processor_patch else 0, out.ctypes.data, err, 1024)
    if rc != 0:
        raise FoamError(err.value.decode())
    return {"initialResidual": out[0], "finalResidual": out[1], "nIterations": int(out[2]),
            "converged": bool(out[3])}
