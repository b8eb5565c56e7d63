"""cufoam_gb300 -- GB300-native sparse iterative solves for OpenFOAM LDU matrices.

The Python layer mirrors the reference's plugin surface: eight
``lduMatrix::solver`` classes selected by name (``cuFoamCG``, ``cuFoamBiCG``,
``cuFoamJacobi``, ``cuFoamMR``, ``cuFoamMRJacobi``, ``cuFoamMRS``,
``cuFoamJMR``, ``cuFoamRichardson``), each with
``solve(psi, source, cmpt=0) -> SolverPerformance`` updating ``psi`` in
place (cuFoamCG/cuFoamCG.H:8-31, cuFoamCG/cuFoamCG.C:38-90).  All work
happens in the C-ABI library ``libcufoam_gb300.so`` (hand-written sm_103a
kernels); arrays may be numpy (host) or CUDA torch tensors (device).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi
from ._capi import (CF_BICG, CF_CG, CF_JACOBI, CF_JMR, CF_MR, CF_MRJACOBI, CF_MRS,
                    CF_RICHARDSON, CF_PCG, CufoamError)

__all__ = ["Context", "LduMatrix", "SolverPerformance", "New", "solver_names",
           "cuFoamCG", "cuFoamBiCG", "cuFoamJacobi", "cuFoamMR", "cuFoamMRJacobi",
           "cuFoamMRS", "cuFoamJMR", "cuFoamRichardson", "cuFoamPCG", "CufoamError", "CsrMatrix",
           "read_csr", "save_csr", "read_vector", "save_vector"]


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _ptr(a, dtype, name):
    """(pointer, memory kind, keepalive) of a numpy array or CUDA tensor."""
    if a is None:
        return None, None, None
    if _is_torch(a):
        import torch
        want = {np.float64: torch.float64, np.int32: torch.int32, np.float32: torch.float32}[dtype]
        if a.dtype != want or not a.is_contiguous():
            raise TypeError(f"{name}: expected a contiguous {want} tensor")
        if a.is_cuda:
            return a.data_ptr(), _capi.CF_MEM_DEVICE, a
        a = a.numpy()
    arr = np.asarray(a)
    if arr.dtype != dtype or not arr.flags["C_CONTIGUOUS"]:
        arr = np.ascontiguousarray(arr, dtype=dtype)
    return arr.ctypes.data, _capi.CF_MEM_HOST, arr


class Context:
    """A CUDA device plus the workspace, stream and cached loop graphs the
    library reuses across solves."""

    def __init__(self, device: int = 0):
        self._lib = _capi.load()
        h = C.c_void_p()
        st = self._lib.cf_context_create(int(device), C.byref(h))
        if st != 0:
            raise CufoamError(st, f"cf_context_create(device={device}) failed")
        self._h = h
        self.device = int(device)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cf_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def last_error(self) -> str:
        return self._lib.cf_context_last_error(self._h).decode()

    def check(self, st: int, what: str) -> None:
        if st != 0:
            raise CufoamError(st, f"{what}: {self.last_error()}")

    def set_stream(self, stream) -> None:
        """Order the library's work on `stream` (a torch.cuda.Stream, a raw
        cudaStream_t as int, or None for a private stream).  Torch's default
        stream (handle 0) is the legacy default stream (cudaStreamLegacy)."""
        if stream is None:
            raw = None
        else:
            raw = getattr(stream, "cuda_stream", stream)
            if raw == 0:
                raw = 1   # cudaStreamLegacy
        self.check(self._lib.cf_context_set_stream(self._h, C.c_void_p(raw) if raw else None),
                   "set_stream")

    def device_info(self) -> dict:
        info = _capi.cf_device_info()
        self.check(self._lib.cf_device_query(self._h, C.byref(info)), "device_query")
        return {"device": info.device, "sm_count": info.sm_count,
                "cc": (info.cc_major, info.cc_minor),
                "max_threads_per_sm": info.max_threads_per_sm,
                "reference_grid": info.reference_grid, "l2_bytes": info.l2_bytes,
                "global_mem_bytes": info.global_mem_bytes, "name": info.name.decode()}


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _ldu_view(n, diag, lower, upper, lower_addr, upper_addr, losort=None, losort_start=None,
              owner_start=None):
    keep = []
    parts = {}
    mem = None
    for nm, arr, dt in (("diag", diag, np.float64), ("lower", lower, np.float64),
                        ("upper", upper, np.float64), ("lower_addr", lower_addr, np.int32),
                        ("upper_addr", upper_addr, np.int32), ("losort", losort, np.int32),
                        ("losort_start", losort_start, np.int32),
                        ("owner_start", owner_start, np.int32)):
        p, m, k = _ptr(arr, dt, nm)
        parts[nm] = p
        if k is not None:
            keep.append(k)
            if mem is None:
                mem = m
            elif m != mem:
                raise ValueError("LDU arrays must all be host arrays or all CUDA tensors")
    nf = int(np.asarray(lower).shape[0]) if not _is_torch(lower) else int(lower.shape[0])
    v = _capi.cf_ldu_view(n_cells=int(n), n_faces=nf, memory=mem or 0, **parts)
    return v, keep


class LduMatrix:
    """An OpenFOAM lduMatrix resident on the GPU as the reference's CSR
    (converted on the device, gis/ldu2csr.h:7-40)."""

    def __init__(self, n_cells, diag, lower, upper, lower_addr, upper_addr, losort=None,
                 losort_start=None, owner_start=None, context: Context | None = None):
        self.ctx = context or default_context()
        self._lib = self.ctx._lib
        v, keep = _ldu_view(n_cells, diag, lower, upper, lower_addr, upper_addr, losort,
                            losort_start, owner_start)
        h = C.c_void_p()
        self.ctx.check(self._lib.cf_matrix_create_ldu(self.ctx.handle, C.byref(v), C.byref(h)),
                       "cf_matrix_create_ldu")
        self._h = h
        self.n = int(n_cells)
        self.n_faces = v.n_faces
        self._set_symmetry(lambda: _same(lower, upper))

    @classmethod
    def from_ldu(cls, ldu, context: Context | None = None, with_addressing: bool = False):
        """From any object with n, diag, lower, upper, lower_addr, upper_addr
        (e.g. the oracle's LDU); optionally passing lduAddressing arrays."""
        extra = {}
        if with_addressing:
            ls, lst, ost = ldu.addressing()
            extra = dict(losort=ls, losort_start=lst, owner_start=ost)
        return cls(ldu.n, ldu.diag, ldu.lower, ldu.upper, ldu.lower_addr, ldu.upper_addr,
                   context=context, **extra)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cf_matrix_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _set_symmetry(self, fn) -> None:
        # decided on the first symmetric() call: comparing the coefficient
        # arrays costs more than a solve's upload, and most callers never ask
        self._symmetric = None
        self._sym_fn = fn

    def symmetric(self) -> bool:
        """lduMatrix::symmetric(): no separate upper coefficients."""
        if self._symmetric is None:
            self._symmetric = bool(self._sym_fn())
            self._sym_fn = None
        return self._symmetric

    def shape(self):
        n, f, z = C.c_int32(), C.c_int32(), C.c_int64()
        self._lib.cf_matrix_shape(self._h, C.byref(n), C.byref(f), C.byref(z))
        return n.value, f.value, z.value

    _FORMATS = {"auto": 0, "csr": 1, "sell": 2, "sell8": 3, "sell16": 4}

    def set_format(self, fmt: str) -> None:
        """Storage the fast kernels read: "auto" (SELL-32 when the padding
        stays within 20% of nnz, else CSR; SELL-32 with one-byte column
        codes when the pattern has at most 32 distinct offsets col - row,
        else 16-bit column deltas when every |col - row| <= 32767), "csr",
        "sell" (32-bit columns), "sell8" (one-byte codes; raises for a
        pattern with more offsets) or "sell16" (16-bit deltas; raises for a
        pattern with a larger offset)."""
        self.ctx.check(self._lib.cf_matrix_set_format(self._h, self._FORMATS[fmt]),
                       "cf_matrix_set_format")

    def format(self):
        """(format the fast kernels use, stored entries incl. padding)."""
        f, z = C.c_int32(), C.c_int64()
        self.ctx.check(self._lib.cf_matrix_format(self._h, C.byref(f), C.byref(z)), "cf_matrix_format")
        return {1: "csr", 2: "sell", 3: "sell8", 4: "sell16"}[f.value], z.value

    def update_values(self, diag, lower, upper) -> None:
        pd, m1, k1 = _ptr(diag, np.float64, "diag")
        pl, m2, k2 = _ptr(lower, np.float64, "lower")
        pu, m3, k3 = _ptr(upper, np.float64, "upper")
        if len({m1, m2, m3}) != 1:
            raise ValueError("coefficients must all be host arrays or all CUDA tensors")
        self.ctx.check(self._lib.cf_matrix_update_values(self._h, pd, pl, pu, m1),
                       "cf_matrix_update_values")
        self._set_symmetry(lambda: _same(lower, upper))

    def to_csr(self, transpose: bool = False):
        n, _, nnz = self.shape()
        ro = np.empty(n + 1, np.int32)
        cols = np.empty(nnz, np.int32)
        vals = np.empty(nnz, np.float64)
        self.ctx.check(self._lib.cf_matrix_export_csr(self._h, int(transpose), ro.ctypes.data,
                                                      cols.ctypes.data, vals.ctypes.data, 0),
                       "cf_matrix_export_csr")
        return ro, cols, vals

    def spmv(self, x, transpose: bool = False, row_order: str = "reference", out=None):
        """y = A x (or A^T x); row_order "reference" sums rows in the
        reference's 8-lane order, "fast" as one FMA chain.  With a CUDA
        tensor `out` (and x on the device) the product is only enqueued on
        the context's stream (no synchronisation)."""
        px, mx, kx = _ptr(x, np.float64, "x")
        if out is not None:
            po, mo, _ = _ptr(out, np.float64, "out")
            if mx != _capi.CF_MEM_DEVICE or mo != _capi.CF_MEM_DEVICE:
                raise ValueError("out= needs x and out on the device")
            self.ctx.check(self._lib.cf_spmv_async(self._h, int(transpose), px, po, _REDUCE[row_order]),
                           "cf_spmv_async")
            return out
        if mx == _capi.CF_MEM_DEVICE:
            import torch
            y = torch.empty_like(kx)
            py = y.data_ptr()
        else:
            y = np.empty(self.n)
            py = y.ctypes.data
        self.ctx.check(self._lib.cf_spmv(self._h, int(transpose), px, py, mx, _REDUCE[row_order]),
                       "cf_spmv")
        return y

    def norm_factor(self, source, psi, norm_type: str = "reference",
                    reduction: str = "fast") -> float:
        pb, mb, kb = _ptr(source, np.float64, "source")
        px, mx, kx = _ptr(psi, np.float64, "psi")
        if mb != mx:
            raise ValueError("source and psi must live in the same memory")
        out = C.c_double()
        self.ctx.check(self._lib.cf_norm_factor(
            self._h, pb, px, mb, _NORM[norm_type], _REDUCE[reduction], C.byref(out)),
            "cf_norm_factor")
        return out.value


class CsrMatrix(LduMatrix):
    """A square matrix given in CSR form (host arrays or CUDA tensors),
    e.g. read from the reference's file formats (`read_csr`).  Solves,
    SpMV and normFactor work as for an LduMatrix; coefficient updates and
    adjoint gradients need the LDU form.  `symmetric()` is the numerical
    symmetry of the given arrays (it selects the symmetric solver table)."""

    def __init__(self, n, row_offsets, cols, vals, context: Context | None = None):
        self.ctx = context or default_context()
        self._lib = self.ctx._lib
        pr, m1, kr = _ptr(row_offsets, np.int32, "row_offsets")
        pc, m2, kc = _ptr(cols, np.int32, "cols")
        pv, m3, kv = _ptr(vals, np.float64, "vals")
        if len({m1, m2, m3}) != 1:
            raise ValueError("CSR arrays must all be host arrays or all CUDA tensors")
        nnz = int(kv.shape[0])
        h = C.c_void_p()
        self.ctx.check(self._lib.cf_matrix_create_csr(self.ctx.handle, int(n), nnz, pr, pc, pv, m1,
                                                      C.byref(h)), "cf_matrix_create_csr")
        self._h = h
        self.n = int(n)
        self.n_faces = -1
        self._pattern = (row_offsets, cols)
        self._set_symmetry(lambda: _csr_symmetric(n, row_offsets, cols, vals))

    def update_values(self, diag, lower, upper) -> None:
        raise NotImplementedError("a CSR matrix has no LDU coefficients (use update_csr_values)")

    def update_csr_values(self, vals) -> None:
        """New values on the same pattern (vals[nnz], host array or CUDA
        tensor, in the entry order the matrix was created with)."""
        pv, mv, kv = _ptr(vals, np.float64, "vals")
        self.ctx.check(self._lib.cf_matrix_update_csr_values(self._h, pv, mv), "cf_matrix_update_csr_values")
        ro, cols = self._pattern
        self._set_symmetry(lambda: _csr_symmetric(self.n, ro, cols, kv))


def _csr_symmetric(n, ro, cols, vals) -> bool:
    to_np = lambda a: a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
    ro, cols, vals = to_np(ro), to_np(cols), to_np(vals)
    rows = np.repeat(np.arange(n), np.diff(ro))
    a = sorted(zip(rows.tolist(), cols.tolist(), vals.tolist()))
    b = sorted(zip(cols.tolist(), rows.tolist(), vals.tolist()))
    return a == b


# ---------------------------------------------------------------------------
# the reference's file formats (gis/SparseSystem/SparseCPU.h)
# ---------------------------------------------------------------------------
def _file_lib():
    return _capi.load()


def _file_check(rc, what):
    if rc != _capi.CF_OK:
        msg = _file_lib().cf_file_last_error().decode()
        raise CufoamError(rc, f"{what}: {msg}")


def read_csr(path: str):
    """(rows, cols, row_offsets, col_indices, values) of a Rutherford-Boeing
    file (name ending in .rb) or of the reference's binary CSR file."""
    L = _file_lib()
    r, c, z = C.c_int32(), C.c_int32(), C.c_int64()
    _file_check(L.cf_csr_file_info(path.encode(), C.byref(r), C.byref(c), C.byref(z)), "cf_csr_file_info")
    ro = np.empty(r.value + 1, np.int32)
    ci = np.empty(max(z.value, 1), np.int32)
    va = np.empty(max(z.value, 1), np.float64)
    _file_check(L.cf_csr_file_read(path.encode(), ro.ctypes.data, ci.ctypes.data, va.ctypes.data),
                "cf_csr_file_read")
    return r.value, c.value, ro, ci[:z.value], va[:z.value]


def save_csr(path: str, rows: int, cols: int, row_offsets, col_indices, values) -> None:
    """The reference's binary CSR file (CPU::SparseCSR::save)."""
    ro = np.ascontiguousarray(row_offsets, np.int32)
    ci = np.ascontiguousarray(col_indices, np.int32)
    va = np.ascontiguousarray(values, np.float64)
    _file_check(_file_lib().cf_csr_file_save(path.encode(), int(rows), int(cols), int(va.shape[0]),
                                             ro.ctypes.data, ci.ctypes.data, va.ctypes.data),
                "cf_csr_file_save")


def read_vector(path: str) -> np.ndarray:
    """A Matrix Market array file (.mtx) or the reference's binary vector."""
    L = _file_lib()
    n = C.c_int32()
    _file_check(L.cf_vector_file_info(path.encode(), C.byref(n)), "cf_vector_file_info")
    v = np.empty(max(n.value, 1))
    _file_check(L.cf_vector_file_read(path.encode(), v.ctypes.data), "cf_vector_file_read")
    return v[:n.value]


def save_vector(path: str, values) -> None:
    """The reference's binary vector file (CPU::Vector::save)."""
    v = np.ascontiguousarray(values, np.float64)
    _file_check(_file_lib().cf_vector_file_save(path.encode(), int(v.shape[0]), v.ctypes.data),
                "cf_vector_file_save")


def _same(a, b) -> bool:
    if a is b:
        return True
    try:
        if _is_torch(a) or _is_torch(b):
            import torch
            return bool(torch.equal(a, b))
        return bool(np.array_equal(np.asarray(a), np.asarray(b)))
    except Exception:
        return False


_NORM = {"reference": _capi.CF_NORM_REFERENCE_L2, "L2": _capi.CF_NORM_REFERENCE_L2,
         "openfoam": _capi.CF_NORM_OPENFOAM_L1, "L1": _capi.CF_NORM_OPENFOAM_L1}
# "auto" (the default): the reference order for BiCG, the fast one for the others
_REDUCE = {"fast": _capi.CF_REDUCE_FAST, "reference": _capi.CF_REDUCE_REFERENCE,
           "auto": _capi.CF_REDUCE_AUTO}
_PREC = {"FP64": _capi.CF_PREC_FP64, "fp64": _capi.CF_PREC_FP64,
         "mixed": _capi.CF_PREC_MIXED}


@dataclass
class SolverPerformance:
    """OpenFOAM's solverPerformance (solver name, field name, initial and
    final residual, iteration count) plus diagnostics.  Residuals are
    normalised by normFactor as OpenFOAM reports them; the *_abs fields are
    the absolute ||r||_2 values libGIS records."""
    solver_name: str
    field_name: str
    initial_residual: float
    final_residual: float
    n_iterations: int
    converged: bool
    status: int
    norm_factor: float
    initial_residual_abs: float
    final_residual_abs: float
    solve_ms: float
    omega: float = 0.0
    n_outer: int = 0
    history: np.ndarray | None = field(default=None, repr=False)
    kernel_ms: tuple = (0.0, 0.0, 0.0, 0.0)        # spmv, update, prep, set-up
    kernel_launches: tuple = (0, 0, 0, 0)

    @property
    def status_name(self) -> str:
        return _capi.status_string(self.status)


class LduSolver:
    """Base of the eight plugins: mirrors lduMatrix::solver (field name,
    matrix, controls dictionary with tolerance / relTol / maxIter / minIter)
    and its solve(psi, source, cmpt) -> solverPerformance."""
    type_name = "lduSolver"
    kind = -1
    symmetric_table = True
    asymmetric_table = True

    def __init__(self, field_name: str, matrix: LduMatrix, controls: dict | None = None,
                 interfaces=None):
        """`interfaces` (a decomposed.ProcessorInterfaces): this matrix is
        one subdomain of a decomposed case, coupled to the others through
        processor patches as OpenFOAM's interfaceBouCoeffs + interfaces
        constructor arguments describe them (cf_solve_decomposed)."""
        self.field_name = field_name
        self.matrix = matrix
        self.controls = dict(controls or {})
        self.interfaces = interfaces

    def _controls(self, memory: int, history_capacity: int):
        c = _capi.cf_controls()
        self.matrix._lib.cf_controls_init(C.byref(c))
        d = self.controls
        c.tolerance = float(d.get("tolerance", 1e-6))
        c.rel_tol = float(d.get("relTol", 0.0))
        c.max_iter = int(d.get("maxIter", 1000))
        c.min_iter = int(d.get("minIter", 0))
        c.precision = _PREC[d.get("precision", "FP64")]
        c.reduction = _REDUCE[d.get("reduction", "auto")]
        c.norm_type = _NORM[d.get("normType", "reference")]
        c.memory = memory
        c.bicg_int_bound = float(d.get("intBound", 1e-10))
        c.richardson_omega = float(d.get("omega", 0.0))
        c.power_max_steps = int(d.get("powerMaxSteps", 30))
        c.mixed_max_outer = int(d.get("maxRefinements", 50))
        c.mixed_inner_rtol = float(d.get("innerRelTol", 0.0))   # 0: the solver's default
        c.mixed_inner_max = int(d.get("innerMaxIter", 0))
        c.use_graph = int(d.get("useGraph", 1))
        c.time_limit_s = float(d.get("timeLimit", 0.0))
        c.profile_kernels = int(d.get("profileKernels", 0))
        c.transpose = int(d.get("transpose", 0))
        return c

    def solve(self, psi, source, cmpt: int = 0, history: int = 0,
              transpose: bool = False) -> SolverPerformance:
        """Solve matrix * psi = source, updating psi in place.  `history`
        > 0 returns up to that many absolute residuals per step; `transpose`
        solves the adjoint system matrix^T psi = source."""
        px, mx, kx = _ptr(psi, np.float64, "psi")
        pb, mb, kb = _ptr(source, np.float64, "source")
        if mx != mb:
            raise ValueError("psi and source must both be host arrays or both CUDA tensors")
        if mx == _capi.CF_MEM_HOST and kx is not psi:
            raise TypeError("psi must be a C-contiguous float64 array (it is updated in place)")
        if len(psi) != self.matrix.n or len(source) != self.matrix.n:
            raise ValueError("psi/source length does not match the matrix")
        hist = np.zeros(history) if history > 0 else None
        c = self._controls(mx, history)
        if transpose:
            c.transpose = 1
        if hist is not None:
            c.history = hist.ctypes.data
            c.history_capacity = history
        perf = _capi.cf_perf()
        if mx == _capi.CF_MEM_DEVICE:
            import torch
            self.matrix.ctx.set_stream(torch.cuda.current_stream(kx.device))
        if self.interfaces is None:
            st = self.matrix._lib.cf_solve(self.matrix.handle, self.kind, C.byref(c), pb, px,
                                           C.byref(perf))
        else:
            ci, cc = self.interfaces.as_c()
            comm = self.interfaces.comm
            comm.error = None
            st = self.matrix._lib.cf_solve_decomposed(self.matrix.handle, self.kind, C.byref(c),
                                                      C.byref(ci), C.byref(cc), pb, px, C.byref(perf))
            if comm.error is not None:
                raise comm.error
        self.matrix.ctx.check(st, f"{self.type_name}::solve")
        h = hist[:perf.history_length].copy() if hist is not None else None
        return SolverPerformance(
            self.type_name, self.field_name, perf.initial_residual, perf.final_residual,
            perf.n_iterations, perf.status == _capi.CF_OK, perf.status, perf.norm_factor,
            perf.initial_residual_abs, perf.final_residual_abs, perf.solve_ms, perf.omega,
            perf.n_outer, h, tuple(perf.kernel_ms), tuple(perf.kernel_launches))


def _plugin(name, kind, sym=True, asym=True):
    cls = type(name, (LduSolver,), {"type_name": name, "kind": kind, "symmetric_table": sym,
                                    "asymmetric_table": asym,
                                    "__doc__": f"The {name} plugin (fvSolution `solver {name};`)."})
    return cls


# Registration tables: CG and Richardson are symmetric-only
# (cuFoamCG/cuFoamCG.C:14-15, cuFoamRichardson/cuFoamRichardson.C:11-12); the
# others register for both (e.g. cuFoamBiCG/cuFoamBiCG.C:11-16).
cuFoamCG = _plugin("cuFoamCG", CF_CG, True, False)
cuFoamBiCG = _plugin("cuFoamBiCG", CF_BICG)
cuFoamJacobi = _plugin("cuFoamJacobi", CF_JACOBI)
cuFoamMR = _plugin("cuFoamMR", CF_MR)
cuFoamMRJacobi = _plugin("cuFoamMRJacobi", CF_MRJACOBI)
cuFoamMRS = _plugin("cuFoamMRS", CF_MRS)
cuFoamJMR = _plugin("cuFoamJMR", CF_JMR)
cuFoamRichardson = _plugin("cuFoamRichardson", CF_RICHARDSON, True, False)
# Jacobi-preconditioned CG: no reference counterpart (the reference's
# roadmap, README.md:71-73); symmetric matrices, like cuFoamCG
cuFoamPCG = _plugin("cuFoamPCG", CF_PCG, True, False)

_TABLE = {c.type_name: c for c in (cuFoamCG, cuFoamBiCG, cuFoamJacobi, cuFoamMR,
                                   cuFoamMRJacobi, cuFoamMRS, cuFoamJMR, cuFoamRichardson,
                                   cuFoamPCG)}


def solver_names(symmetric: bool = True) -> list[str]:
    return sorted(n for n, c in _TABLE.items()
                  if (c.symmetric_table if symmetric else c.asymmetric_table))


def New(field_name: str, matrix: LduMatrix, controls: dict) -> LduSolver:
    """Run-time selection by name, like lduMatrix::solver::New: the
    `solver` entry of `controls` picks the plugin from the symmetric or the
    asymmetric table according to matrix.symmetric()."""
    name = controls.get("solver")
    cls = _TABLE.get(name)
    sym = matrix.symmetric()
    if cls is None or not (cls.symmetric_table if sym else cls.asymmetric_table):
        kind = "symmetric" if sym else "asymmetric"
        raise KeyError(f"Unknown {kind} matrix solver {name}; valid solvers are "
                       f"{solver_names(sym)}")
    return cls(field_name, matrix, controls)
