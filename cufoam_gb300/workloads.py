"""Seeded synthetic LDU workloads (inputs for benchmarks, tests and examples).

Structured 5/7-point grids in OpenFOAM upper-triangular face order (faces
sorted by owner, then neighbour; the faces of cell c go to c+1, c+nx,
c+nx*ny), with:

* ``grid_const``     -- Poisson, diag 4 (2-D) / 6 (3-D), off-diagonals -1,
                        Dirichlet-0 walls folded into the diagonal;
* ``grid_lognormal`` -- face coefficients k ~ lognormal(0,1), lower = upper
                        = -k, diag = sum of k incl. a lognormal wall term per
                        boundary face (SPD);
* ``grid_convdiff``  -- upwind convection-diffusion with a divergence-free
                        smooth random velocity scaled to a maximum cell
                        Peclet number (non-symmetric M-matrix);
* ``grid_grf`` + ``diffusion_from_cells`` -- diffusion with conductivity
                        exp(Gaussian random field);
* ``uniform``, ``normal``, ``permutation``, ``permute_ldu``.

All values come from ``workloads.c`` (splitmix64 + correctly rounded
arithmetic only), so every host produces identical bytes for a seed.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "workloads.c")
LIB = os.path.join(HERE, "_build", "libcufoam_workloads.so")

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp",
                               "-ffp-contract=off", "-Wall", SRC, "-o", tmp, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        for fn in ("wl_exp", "wl_log", "wl_sin", "wl_cos"):
            getattr(L, fn).restype = C.c_double
            getattr(L, fn).argtypes = [C.c_double]
        L.wl_fill_uniform.argtypes = [C.c_uint64, C.c_double, C.c_double, _dp, C.c_int64]
        L.wl_fill_normal.argtypes = [C.c_uint64, _dp, C.c_int64]
        L.wl_permutation.argtypes = [C.c_uint64, C.c_int32, _ip]
        L.wl_grid_n_faces.restype = C.c_int64
        L.wl_grid_n_faces.argtypes = [C.c_int32] * 3
        L.wl_grid_addressing.argtypes = [C.c_int32] * 3 + [_ip, _ip]
        L.wl_grid_const.argtypes = [C.c_int32] * 3 + [C.c_double, C.c_double, _dp, _dp, _dp]
        L.wl_grid_lognormal.argtypes = [C.c_int32] * 3 + [C.c_uint64, _dp, _dp, _dp]
        L.wl_grid_convdiff.argtypes = [C.c_int32] * 3 + [C.c_uint64, C.c_double, _dp, _dp, _dp, _dp]
        L.wl_grid_grf.argtypes = [C.c_int32] * 3 + [C.c_uint64, C.c_double, _dp]
        L.wl_grid_diffusion_from_cells.argtypes = [C.c_int32] * 3 + [_dp] * 6
        _lib = L
    return _lib


@dataclass
class LDU:
    """An OpenFOAM lduMatrix: diag[n], lower[F], upper[F] and the face
    addressing lowerAddr (owner) / upperAddr (neighbour), faces sorted by
    owner then neighbour."""
    n: int
    diag: np.ndarray
    lower: np.ndarray
    upper: np.ndarray
    lower_addr: np.ndarray
    upper_addr: np.ndarray
    _addr: tuple | None = field(default=None, repr=False)

    @property
    def n_faces(self) -> int:
        return int(self.lower.shape[0])

    def addressing(self):
        """(losort, losortStart, ownerStart) with OpenFOAM's semantics:
        faces stably sorted by neighbour, and first-position lookups."""
        if self._addr is None:
            ua = np.asarray(self.upper_addr)
            la = np.asarray(self.lower_addr)
            losort = np.argsort(ua, kind="stable").astype(np.int32)
            cells = np.arange(self.n + 1)
            lstart = np.searchsorted(ua[losort], cells, side="left").astype(np.int32)
            ostart = np.searchsorted(la, cells, side="left").astype(np.int32)
            self._addr = (losort, lstart, ostart)
        return self._addr

    def transposed(self) -> "LDU":
        """A^T in LDU form: lower and upper swapped, same addressing."""
        return LDU(self.n, self.diag, self.upper, self.lower, self.lower_addr,
                   self.upper_addr, self._addr)

    def nbytes(self) -> int:
        return sum(int(np.asarray(a).nbytes) for a in
                   (self.diag, self.lower, self.upper, self.lower_addr, self.upper_addr))


def uniform(seed: int, n: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    out = np.empty(n, np.float64)
    lib().wl_fill_uniform(seed, lo, hi, out, n)
    return out


def normal(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    lib().wl_fill_normal(seed, out, n)
    return out


def permutation(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.int32)
    lib().wl_permutation(seed, n, out)
    return out


def n_faces(nx: int, ny: int, nz: int = 1) -> int:
    return int(lib().wl_grid_n_faces(nx, ny, nz))


def grid_addressing(nx: int, ny: int, nz: int = 1):
    nf = n_faces(nx, ny, nz)
    la = np.empty(nf, np.int32)
    ua = np.empty(nf, np.int32)
    lib().wl_grid_addressing(nx, ny, nz, la, ua)
    return la, ua


def _empty(nx, ny, nz):
    la, ua = grid_addressing(nx, ny, nz)
    n = nx * ny * nz
    return la, ua, np.empty(n), np.empty(la.shape[0]), np.empty(la.shape[0])


def grid_const(nx: int, ny: int, nz: int = 1, diag_value: float | None = None,
               off_value: float = -1.0) -> LDU:
    if diag_value is None:
        diag_value = 4.0 if nz == 1 else 6.0
    la, ua, d, lo, up = _empty(nx, ny, nz)
    lib().wl_grid_const(nx, ny, nz, diag_value, off_value, d, lo, up)
    return LDU(nx * ny * nz, d, lo, up, la, ua)


def grid_lognormal(nx: int, ny: int, nz: int, seed: int) -> LDU:
    la, ua, d, lo, up = _empty(nx, ny, nz)
    lib().wl_grid_lognormal(nx, ny, nz, seed, d, lo, up)
    return LDU(nx * ny * nz, d, lo, up, la, ua)


def grid_convdiff(nx: int, ny: int, nz: int, seed: int, pe_max: float = 10.0):
    la, ua, d, lo, up = _empty(nx, ny, nz)
    stats = np.zeros(3)
    lib().wl_grid_convdiff(nx, ny, nz, seed, pe_max, d, lo, up, stats)
    return LDU(nx * ny * nz, d, lo, up, la, ua), {
        "pe_min": float(stats[0]), "pe_max": float(stats[1]), "frac_below_0.1": float(stats[2])}


def grid_grf(nx: int, ny: int, nz: int, seed: int, corr_len: float = 8.0) -> np.ndarray:
    g = np.empty(nx * ny * nz)
    lib().wl_grid_grf(nx, ny, nz, seed, corr_len, g)
    return g


def diffusion_from_cells(nx: int, ny: int, nz: int, g: np.ndarray):
    """(LDU, k_face, k_wall_sum): face conductivity exp(mean of the two
    cells' g), wall faces exp(g_cell) folded into the diagonal."""
    la, ua, d, lo, up = _empty(nx, ny, nz)
    kf = np.empty(la.shape[0])
    kb = np.empty(nx * ny * nz)
    lib().wl_grid_diffusion_from_cells(nx, ny, nz, np.ascontiguousarray(g, np.float64), kf, kb,
                                       d, lo, up)
    return LDU(nx * ny * nz, d, lo, up, la, ua), kf, kb


def permute_ldu(ldu: LDU, perm: np.ndarray) -> LDU:
    """P A P^T: cell i becomes cell perm[i]; faces rebuilt in
    upper-triangular order, swapping lower/upper where the ends swap."""
    perm = np.ascontiguousarray(perm, np.int32)
    a = perm[ldu.lower_addr]
    b = perm[ldu.upper_addr]
    swap = a > b
    own = np.where(swap, b, a).astype(np.int32)
    nbr = np.where(swap, a, b).astype(np.int32)
    lo = np.where(swap, ldu.upper, ldu.lower)
    up = np.where(swap, ldu.lower, ldu.upper)
    order = np.lexsort((nbr, own))
    diag = np.empty_like(ldu.diag)
    diag[perm] = ldu.diag
    return LDU(ldu.n, diag, np.ascontiguousarray(lo[order]), np.ascontiguousarray(up[order]),
               np.ascontiguousarray(own[order]), np.ascontiguousarray(nbr[order]))
