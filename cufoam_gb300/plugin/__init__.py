"""Access to the C++ plugin layer (cuFoamGB300.{H,C}) compiled against the
minifoam stand-in: ``foam_solve`` runs a plugin exactly as OpenFOAM would
(lduMatrix::solver::New by name, then solve(psi, source, cmpt));
``foam_solve_decomposed`` runs it on one subdomain of a parallel run, the
stand-in's Pstream carried by ``torch.distributed`` (``ParallelRun``)."""
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
        L.cuFoamGB300_coupled_builds.restype = C.c_long
        L.cuFoamGB300_coupled_builds.argtypes = []
        # mf_solve_coupled without its processor flag, after a slot number
        L.mf_solve_coupled_reused.restype = C.c_int
        L.mf_solve_coupled_reused.argtypes = [C.c_int] + list(L.mf_solve_coupled.argtypes[:21]) + \
            [C.c_void_p, C.c_char_p, C.c_int]
        L.mf_set_transport.restype = None
        L.mf_set_transport.argtypes = [C.c_void_p]
        L.mf_solve_decomposed.restype = C.c_int
        L.mf_solve_decomposed.argtypes = list(L.mf_solve.argtypes[:16]) + \
            [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
        L.mf_processor_comm_check.restype = C.c_int
        L.mf_processor_comm_check.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                              C.c_int, C.c_char_p, C.c_int]
        _lib = L
    return _lib


def matrix_builds() -> int:
    """Device matrices the plugin has built so far (its cache misses)."""
    return int(lib().cuFoamGB300_matrix_builds())


def coupled_builds() -> int:
    """Coupled (cyclic-patch) matrices the plugin has built so far (the
    misses of their cache)."""
    return int(lib().cuFoamGB300_coupled_builds())


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
        if reuse_addressing is not None and not processor_patch:
            rc = lib().mf_solve_coupled_reused(int(reuse_addressing), solver.encode(), ldu.n, lo.shape[0],
                                               d.ctypes.data, None if symmetric else lo.ctypes.data,
                                               up.ctypes.data, la.ctypes.data, ua.ctypes.data, b.ctypes.data,
                                               psi.ctypes.data, tolerance, rel_tol, max_iter, len(keys), ck,
                                               cv, int(fa.shape[0]), fa.ctypes.data, fb.ctypes.data,
                                               ca.ctypes.data, cb.ctypes.data, out.ctypes.data, err, 1024)
        else:
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


# ---------------------------------------------------------------------------
# parallel runs: minifoam's Pstream over torch.distributed
# ---------------------------------------------------------------------------
_COMPLETE_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                           C.POINTER(C.c_int32), C.POINTER(C.c_void_p), C.POINTER(C.c_int64))
_ALLREDUCE_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.POINTER(C.c_double), C.c_int32)


class _Transport(C.Structure):
    _fields_ = [("myProcNo", C.c_int32), ("nProcs", C.c_int32), ("user", C.c_void_p),
                ("complete", _COMPLETE_FN), ("allreduceSum", _ALLREDUCE_FN),
                ("allreduceMax", _ALLREDUCE_FN)]


class ParallelRun:
    """A parallel run of the stand-in, carried by this process's
    torch.distributed group (gloo): the plugin's non-blocking processor
    transfers become isend / irecv with their tags, its reductions an
    all-gather summed in rank order (the same bits on every rank, as a
    parallel solver needs).  Use as a context manager around the solves."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.error: BaseException | None = None
        self._complete = _COMPLETE_FN(self._on_complete)
        self._reduce = _ALLREDUCE_FN(self._on_reduce)
        self._max = _ALLREDUCE_FN(self._on_max)
        self._t = _Transport(dist.get_rank(group), dist.get_world_size(group), None,
                             self._complete, self._reduce, self._max)

    def _on_complete(self, _user, n, kind, peer, tag, data, nbytes):
        import torch
        try:
            reqs, keep = [], []
            for i in range(n):
                if nbytes[i] % 8:
                    raise ValueError("transfers of doubles only")
                buf = np.ctypeslib.as_array(C.cast(data[i], C.POINTER(C.c_double)), shape=(nbytes[i] // 8,)) \
                    if nbytes[i] else np.zeros(0)
                t = torch.from_numpy(buf)
                keep.append(t)
                op = self.dist.isend if kind[i] == 0 else self.dist.irecv
                dst = peer[i] if self.group is None else self.dist.get_global_rank(self.group, peer[i])
                reqs.append(op(t, dst, group=self.group, tag=int(tag[i])))
            for r in reqs:
                r.wait()
            return 0
        except BaseException as e:  # noqa: BLE001 -- reported through the status
            self.error = e
            return 1

    def _on_reduce(self, _user, values, count):
        from ..decomposed import ordered_allreduce_sum
        try:
            ordered_allreduce_sum(np.ctypeslib.as_array(values, shape=(count,)), self.group)
            return 0
        except BaseException as e:  # noqa: BLE001
            self.error = e
            return 1

    def _on_max(self, _user, values, count):
        from ..decomposed import ordered_allreduce_max
        try:
            ordered_allreduce_max(np.ctypeslib.as_array(values, shape=(count,)), self.group)
            return 0
        except BaseException as e:  # noqa: BLE001
            self.error = e
            return 1

    def __enter__(self):
        lib().mf_set_transport(C.addressof(self._t))
        return self

    def __exit__(self, *exc):
        lib().mf_set_transport(None)
        return False


def _proc_arrays(sub):
    neighbours = np.array([p.neighbour for p in sub.patches], np.int32)
    sizes = np.array([len(p.face_cells) for p in sub.patches], np.int32)
    cells, coeffs = sub.interface_arrays()
    return neighbours, sizes, np.ascontiguousarray(cells, np.int32), np.ascontiguousarray(coeffs, np.float64)


def foam_solve_decomposed(solver: str, sub, source, psi, tolerance: float = 1e-6, rel_tol: float = 0.0,
                          max_iter: int = 1000, symmetric: bool | None = None, **controls):
    """Run the plugin `solver` on subdomain `sub` (a decomposed.Subdomain)
    of a parallel run (inside ``with ParallelRun():``), its processor
    patches given to the solver as OpenFOAM's processor interfaces; psi
    (this rank's cells) is updated in place.  Returns the solverPerformance
    fields as a dict."""
    if symmetric is None:
        symmetric = np.array_equal(sub.lower, sub.upper)
    d = np.ascontiguousarray(sub.diag, np.float64)
    lo = np.ascontiguousarray(sub.lower, np.float64)
    up = np.ascontiguousarray(sub.upper, np.float64)
    la = np.ascontiguousarray(sub.lower_addr, np.int32)
    ua = np.ascontiguousarray(sub.upper_addr, np.int32)
    b = np.ascontiguousarray(source, np.float64)
    if psi.dtype != np.float64 or not psi.flags["C_CONTIGUOUS"]:
        raise TypeError("psi must be a contiguous float64 array")
    nb, sz, fc, co = _proc_arrays(sub)
    keys = [k.encode() for k in controls]
    vals = [str(v).encode() for v in controls.values()]
    ck = (C.c_char_p * max(1, len(keys)))(*keys)
    cv = (C.c_char_p * max(1, len(vals)))(*vals)
    out = np.zeros(4)
    err = C.create_string_buffer(1024)
    rc = lib().mf_solve_decomposed(solver.encode(), sub.n, lo.shape[0], d.ctypes.data,
                                   None if symmetric else lo.ctypes.data, up.ctypes.data, la.ctypes.data,
                                   ua.ctypes.data, b.ctypes.data, psi.ctypes.data, tolerance, rel_tol,
                                   max_iter, len(keys), ck, cv, len(nb), nb.ctypes.data, sz.ctypes.data,
                                   fc.ctypes.data, co.ctypes.data, out.ctypes.data, err, 1024)
    if rc != 0:
        raise FoamError(err.value.decode())
    return {"initialResidual": out[0], "finalResidual": out[1], "nIterations": int(out[2]),
            "converged": bool(out[3])}


def processor_comm_check(sub, send, values):
    """Drive the plugin's processor-patch callbacks (cuFoamGB300Comm.H)
    once without a solve, inside ``with ParallelRun():``: returns (status,
    recv, sums, maxima) after one exchange of `send` and one sum and one
    maximum of `values` over the ranks."""
    nb, sz, fc, co = _proc_arrays(sub)
    s = np.ascontiguousarray(send, np.float64)
    r = np.zeros(max(1, len(s)))
    v = np.ascontiguousarray(values, np.float64).copy()
    mx = v.copy()
    err = C.create_string_buffer(1024)
    rc = lib().mf_processor_comm_check(len(nb), nb.ctypes.data, sz.ctypes.data, fc.ctypes.data,
                                       co.ctypes.data, s.ctypes.data if len(s) else r.ctypes.data,
                                       r.ctypes.data, len(s), v.ctypes.data, mx.ctypes.data, len(v), err, 1024)
    if rc < 0:
        raise FoamError(err.value.decode())
    return rc, r[:len(s)], v, mx
