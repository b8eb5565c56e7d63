"""ctypes bindings of the C ABI declared in include/cufoam_gb300.h.

The shared library is built in-tree (``cufoam_gb300/_build``).  Loading
fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

CF_OK, CF_NOT_CONVERGED, CF_BREAKDOWN, CF_NONFINITE, CF_BAD_INPUT, CF_CUDA_ERROR, \
    CF_TIMEOUT, CF_NO_DEVICE, CF_UNSUPPORTED, CF_OUT_OF_MEMORY = range(10)
CF_CG, CF_BICG, CF_JACOBI, CF_MR, CF_MRJACOBI, CF_MRS, CF_JMR, CF_RICHARDSON, CF_PCG = range(9)
CF_MEM_HOST, CF_MEM_DEVICE = 0, 1
CF_PREC_FP64, CF_PREC_MIXED = 0, 1
CF_REDUCE_FAST, CF_REDUCE_REFERENCE, CF_REDUCE_AUTO = 0, 1, 2
CF_NORM_REFERENCE_L2, CF_NORM_OPENFOAM_L1 = 0, 1
CF_FORMAT_AUTO, CF_FORMAT_CSR, CF_FORMAT_SELL, CF_FORMAT_SELL_C8, CF_FORMAT_SELL_D16 = 0, 1, 2, 3, 4


class cf_ldu_view(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("n_faces", C.c_int32),
                ("diag", C.c_void_p), ("lower", C.c_void_p), ("upper", C.c_void_p),
                ("lower_addr", C.c_void_p), ("upper_addr", C.c_void_p),
                ("losort", C.c_void_p), ("losort_start", C.c_void_p), ("owner_start", C.c_void_p),
                ("memory", C.c_int32)]


class cf_controls(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("rel_tol", C.c_double),
                ("max_iter", C.c_int32), ("min_iter", C.c_int32),
                ("precision", C.c_int32), ("reduction", C.c_int32),
                ("memory", C.c_int32), ("norm_type", C.c_int32),
                ("bicg_int_bound", C.c_double), ("richardson_omega", C.c_double),
                ("power_max_steps", C.c_int32), ("mixed_max_outer", C.c_int32),
                ("mixed_inner_rtol", C.c_double),
                ("history", C.c_void_p), ("history_capacity", C.c_int32),
                ("use_graph", C.c_int32), ("time_limit_s", C.c_double),
                ("profile_kernels", C.c_int32), ("transpose", C.c_int32),
                ("absolute_tolerance", C.c_int32), ("history_time", C.c_int32),
                ("mixed_inner_max", C.c_int32), ("reserved", C.c_int32 * 3)]


class cf_perf(C.Structure):
    _fields_ = [("initial_residual", C.c_double), ("final_residual", C.c_double),
                ("initial_residual_abs", C.c_double), ("final_residual_abs", C.c_double),
                ("norm_factor", C.c_double), ("true_residual", C.c_double),
                ("omega", C.c_double), ("solve_ms", C.c_double),
                ("n_iterations", C.c_int32), ("n_outer", C.c_int32),
                ("status", C.c_int32), ("history_length", C.c_int32),
                ("kernel_ms", C.c_double * 4), ("kernel_launches", C.c_int32 * 4),
                ("reserved", C.c_int32 * 6)]


# decomposed solves: the caller's exchange / all-reduce (cf_comm)
EXCHANGE_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                          C.c_int32)
ALLREDUCE_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.POINTER(C.c_double), C.c_int32)


class cf_comm(C.Structure):
    _fields_ = [("user", C.c_void_p), ("exchange", EXCHANGE_FN), ("allreduce_sum", ALLREDUCE_FN),
                ("allreduce_max", ALLREDUCE_FN)]


class cf_interfaces(C.Structure):
    _fields_ = [("n_faces", C.c_int32), ("face_cells", C.c_void_p), ("coeffs", C.c_void_p)]


class cf_device_info(C.Structure):
    _fields_ = [("device", C.c_int32), ("sm_count", C.c_int32),
                ("cc_major", C.c_int32), ("cc_minor", C.c_int32),
                ("max_threads_per_sm", C.c_int32), ("reference_grid", C.c_int32),
                ("l2_bytes", C.c_int64), ("global_mem_bytes", C.c_int64),
                ("name", C.c_char * 128)]


_lib = None


def header_functions() -> list[str]:
    """Function names declared in include/*.h (the ABI surface)."""
    names = []
    inc = os.path.join(_build.ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            text = open(os.path.join(inc, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(cf_\w+)\s*\(", text)
    return sorted(set(names))


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load libcufoam_gb300.so (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"{path} is not built; run __graft_entry__.build()")
        _build.build()
    L = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "cf_abi_version": (C.c_int32, []),
        "cf_status_string": (C.c_char_p, [C.c_int32]),
        "cf_solver_from_name": (C.c_int32, [C.c_char_p, C.POINTER(C.c_int32)]),
        "cf_controls_init": (None, [C.POINTER(cf_controls)]),
        "cf_context_create": (C.c_int32, [C.c_int32, C.POINTER(P)]),
        "cf_context_destroy": (None, [P]),
        "cf_context_set_stream": (C.c_int32, [P, P]),
        "cf_context_last_error": (C.c_char_p, [P]),
        "cf_device_query": (C.c_int32, [P, C.POINTER(cf_device_info)]),
        "cf_matrix_create_ldu": (C.c_int32, [P, C.POINTER(cf_ldu_view), C.POINTER(P)]),
        "cf_matrix_update_values": (C.c_int32, [P, P, P, P, C.c_int32]),
        "cf_matrix_destroy": (None, [P]),
        "cf_matrix_shape": (C.c_int32, [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                        C.POINTER(C.c_int64)]),
        "cf_matrix_export_csr": (C.c_int32, [P, C.c_int32, P, P, P, C.c_int32]),
        "cf_matrix_set_format": (C.c_int32, [P, C.c_int32]),
        "cf_matrix_update_csr_values": (C.c_int32, [P, P, C.c_int32]),
        "cf_matrix_create_csr": (C.c_int32, [P, C.c_int32, C.c_int64, P, P, P, C.c_int32, P]),
        "cf_csr_file_info": (C.c_int32, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int64)]),
        "cf_csr_file_read": (C.c_int32, [C.c_char_p, P, P, P]),
        "cf_csr_file_save": (C.c_int32, [C.c_char_p, C.c_int32, C.c_int32, C.c_int64, P, P, P]),
        "cf_vector_file_info": (C.c_int32, [C.c_char_p, C.POINTER(C.c_int32)]),
        "cf_vector_file_read": (C.c_int32, [C.c_char_p, P]),
        "cf_vector_file_save": (C.c_int32, [C.c_char_p, C.c_int32, P]),
        "cf_file_last_error": (C.c_char_p, []),
        "cf_matrix_format": (C.c_int32, [P, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
        "cf_ldu2csr": (C.c_int32, [P, C.POINTER(cf_ldu_view), P, P, P, C.c_int32]),
        "cf_spmv": (C.c_int32, [P, C.c_int32, P, P, C.c_int32, C.c_int32]),
        "cf_spmv_async": (C.c_int32, [P, C.c_int32, P, P, C.c_int32]),
        "cf_norm_factor": (C.c_int32, [P, P, P, C.c_int32, C.c_int32, C.c_int32,
                                       C.POINTER(C.c_double)]),
        "cf_solve": (C.c_int32, [P, C.c_int32, C.POINTER(cf_controls), P, P,
                                 C.POINTER(cf_perf)]),
        "cf_solve_decomposed": (C.c_int32, [P, C.c_int32, C.POINTER(cf_controls),
                                            C.POINTER(cf_interfaces), C.POINTER(cf_comm), P, P,
                                            C.POINTER(cf_perf)]),
        "cf_adjoint_gradients": (C.c_int32, [P, P, P, P, P, P, C.c_int32]),
        "cf_norm_factor_noalloc": (C.c_int32, [C.c_int32, P, P, P, P, P, C.c_int32, P, P]),
    }
    for name, (res, args) in sig.items():
        if not hasattr(L, name):
            continue
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def status_string(code: int) -> str:
    return load().cf_status_string(code).decode()


class CufoamError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{status_string(status)} ({status}): {message}")
        self.status = status
