"""Decomposed cases: one subdomain per rank, coupled through processor patches.

OpenFOAM runs a decomposed case with one process per subdomain; the
subdomains meet at processor patches, and lduMatrix::Amul completes each
rank's product there: after the local product, row ``faceCells[f]`` loses
``interfaceBouCoeffs[f]`` times the neighbouring rank's value of the cell
across face ``f`` (initMatrixInterfaces / updateMatrixInterfaces).  Every
inner product and normFactor sums over all ranks.  The reference takes the
interface lists in its constructors and never uses them
(cuFoamCG/cuFoamCG.C:19-35), so its decomposed runs solve every subdomain
alone; here the coupling is part of the solve (``cf_solve_decomposed``).

This module holds the host side:

* :func:`decompose` splits an LDU matrix by a cell -> rank map into
  subdomains with processor patches (the faces of each patch in ascending
  global face order, which both sides of the patch share, as
  decomposePar's processor patches are ordered alike on both sides);
* :class:`ProcessorComm` moves the patch values between ranks and sums the
  reductions with ``torch.distributed`` (any backend that handles CPU
  tensors, e.g. gloo);
* :class:`ProcessorInterfaces` is what a solver is given (the face cells,
  the coefficients and the communicator), the counterpart of OpenFOAM's
  ``interfaceBouCoeffs`` + ``interfaces`` constructor arguments.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi


@dataclass
class ProcessorPatch:
    """The faces this subdomain shares with one neighbouring subdomain."""
    neighbour: int              # rank on the other side
    face_cells: np.ndarray      # int32 local cell of each face
    coeffs: np.ndarray          # float64 interfaceBouCoeffs: -(global off-diagonal coefficient)
    faces: np.ndarray           # int64 global face index of each face (ascending)


@dataclass
class Subdomain:
    """One rank's part of a decomposed LDU matrix: the cells it owns (global
    indices, ascending), the internal faces among them in local numbering,
    and its processor patches (ordered by neighbour rank)."""
    rank: int
    cells: np.ndarray
    diag: np.ndarray
    lower: np.ndarray
    upper: np.ndarray
    lower_addr: np.ndarray
    upper_addr: np.ndarray
    patches: list = field(default_factory=list)

    @property
    def n(self) -> int:
        return len(self.cells)

    def interface_arrays(self):
        """(face_cells, coeffs) of all patches, patch after patch."""
        if not self.patches:
            return np.zeros(0, np.int32), np.zeros(0, np.float64)
        return (np.concatenate([p.face_cells for p in self.patches]).astype(np.int32),
                np.concatenate([p.coeffs for p in self.patches]).astype(np.float64))


def decompose(n, lower_addr, upper_addr, diag, lower, upper, cell_rank,
              n_ranks: int | None = None) -> list:
    """Split an LDU matrix (OpenFOAM's owner = lower_addr < neighbour =
    upper_addr, faces in upper-triangular order) into subdomains.

    Within a subdomain the cells keep their global order, so the internal
    faces stay in upper-triangular order.  A face whose cells lie on ranks
    r (owner) and s (neighbour) becomes a processor face on both: on r its
    cell is the owner and its coefficient ``-upper[f]`` (row owner, column
    neighbour of the global matrix), on s its cell is the neighbour and its
    coefficient ``-lower[f]``; Amul's ``result -= coeff * ghost`` then
    restores the global product's term."""
    la = np.asarray(lower_addr, dtype=np.int64)
    ua = np.asarray(upper_addr, dtype=np.int64)
    lo = np.asarray(lower, dtype=np.float64)
    up = np.asarray(upper, dtype=np.float64)
    dg = np.asarray(diag, dtype=np.float64)
    cr = np.asarray(cell_rank, dtype=np.int64)
    if len(cr) != n or len(dg) != n:
        raise ValueError("cell_rank and diag must have one entry per cell")
    if len(la) != len(ua) or len(lo) != len(la) or len(up) != len(la):
        raise ValueError("face arrays differ in length")
    if len(la) and (la.min() < 0 or ua.max() >= n or np.any(la >= ua)):
        raise ValueError("faces must have 0 <= owner < neighbour < n")
    if n_ranks is None:
        n_ranks = int(cr.max()) + 1 if n else 0
    if n and (cr.min() < 0 or cr.max() >= n_ranks):
        raise ValueError("cell_rank out of range")
    g2l = np.empty(n, dtype=np.int64)
    subs = []
    ro, rn = cr[la], cr[ua]
    faces = np.arange(len(la), dtype=np.int64)
    for r in range(n_ranks):
        cells = np.flatnonzero(cr == r)
        g2l[cells] = np.arange(len(cells))
        inner = (ro == r) & (rn == r)
        sub = Subdomain(r, cells, dg[cells].copy(), lo[inner].copy(), up[inner].copy(),
                        g2l[la[inner]].astype(np.int32), g2l[ua[inner]].astype(np.int32))
        own = (ro == r) & (rn != r)        # this rank holds the owner
        nbr = (rn == r) & (ro != r)        # this rank holds the neighbour
        for s in sorted(set(rn[own].tolist()) | set(ro[nbr].tolist())):
            fo = faces[own & (rn == s)]
            fn = faces[nbr & (ro == s)]
            f = np.sort(np.concatenate([fo, fn]))
            is_owner = cr[la[f]] == r
            cell = np.where(is_owner, la[f], ua[f])
            coeff = np.where(is_owner, -up[f], -lo[f])
            sub.patches.append(ProcessorPatch(int(s), g2l[cell].astype(np.int32),
                                              coeff.astype(np.float64), f))
        subs.append(sub)
    return subs


def ordered_allreduce_sum(values: np.ndarray, group=None) -> None:
    """values[:] = their sum over the ranks of `group`, added in rank order
    after an all-gather, so that every rank holds the same bits."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(values, dtype=np.float64))
    parts = [torch.empty_like(t) for _ in range(dist.get_world_size(group))]
    dist.all_gather(parts, t, group=group)
    acc = parts[0].clone()
    for q in parts[1:]:
        acc += q
    values[:] = acc.numpy()


def ordered_allreduce_max(values: np.ndarray, group=None) -> None:
    """values[:] = their maximum over the ranks of `group`."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(values, dtype=np.float64))
    parts = [torch.empty_like(t) for _ in range(dist.get_world_size(group))]
    dist.all_gather(parts, t, group=group)
    values[:] = torch.stack(parts).max(dim=0).values.numpy()


class ProcessorComm:
    """Processor-patch exchange and global sums over ``torch.distributed``.

    ``exchange(send, recv)``: for every patch, this rank's values of the
    patch's cells go to the neighbour and the neighbour's values of the
    cells across the same faces come back, in the shared face order.
    ``allreduce_sum(values)``: every rank's values are gathered and added
    in rank order, so all ranks hold bit-identical sums (the solve's
    stopping decisions must agree on every rank); ``allreduce_max`` the
    same with the maximum."""

    def __init__(self, patches, group=None):
        import torch.distributed as dist
        self._dist = dist
        self.group = group
        self.slices = []
        o = 0
        seen = {}
        for p in patches:
            m = len(p.face_cells)
            nb = int(p.neighbour)
            # the k-th patch to a neighbour sends with tag k, so that two
            # patches between the same pair of ranks cannot be confused
            tag = seen.get(nb, 0)
            seen[nb] = tag + 1
            self.slices.append((nb, o, o + m, tag))
            o += m
        self.n_faces = o
        self.error: BaseException | None = None

    def _global(self, r: int) -> int:
        if self.group is None:
            return r
        return self._dist.get_global_rank(self.group, r)

    def exchange(self, send: np.ndarray, recv: np.ndarray) -> None:
        import torch
        dist = self._dist
        reqs = []
        keep = []
        for nb, a, b, tag in self.slices:
            s = torch.from_numpy(np.ascontiguousarray(send[a:b]))
            t = torch.from_numpy(recv[a:b])
            keep += [s, t]
            reqs.append(dist.isend(s, self._global(nb), group=self.group, tag=tag))
            reqs.append(dist.irecv(t, self._global(nb), group=self.group, tag=tag))
        for q in reqs:
            q.wait()

    def allreduce_sum(self, values: np.ndarray) -> None:
        ordered_allreduce_sum(values, self.group)

    def allreduce_max(self, values: np.ndarray) -> None:
        ordered_allreduce_max(values, self.group)

    # ---- the C callbacks -------------------------------------------------
    def as_c(self) -> _capi.cf_comm:
        """A cf_comm whose callbacks call exchange / allreduce_sum; the
        object keeps the callbacks alive.  A Python exception inside a
        callback is kept in ``self.error`` and reported to the library as a
        failure (the solve then ends with CF_BAD_INPUT)."""
        def ex(_user, sp, rp, count):
            try:
                if count != self.n_faces:
                    raise RuntimeError(f"exchange of {count} values, {self.n_faces} expected")
                if count:
                    s = np.ctypeslib.as_array(sp, shape=(count,))
                    r = np.ctypeslib.as_array(rp, shape=(count,))
                    self.exchange(s, r)
                return 0
            except BaseException as e:  # noqa: BLE001 -- reported through the status
                self.error = e
                return 1

        def reducer(method):
            def red(_user, vp, count):
                try:
                    method(np.ctypeslib.as_array(vp, shape=(count,)))
                    return 0
                except BaseException as e:  # noqa: BLE001
                    self.error = e
                    return 1
            return red

        self._c_ex = _capi.EXCHANGE_FN(ex)
        self._c_red = _capi.ALLREDUCE_FN(reducer(self.allreduce_sum))
        self._c_max = _capi.ALLREDUCE_FN(reducer(self.allreduce_max))
        c = _capi.cf_comm()
        c.user = None
        c.exchange = self._c_ex
        c.allreduce_sum = self._c_red
        c.allreduce_max = self._c_max
        return c


class ProcessorInterfaces:
    """The interface arguments of a decomposed solve: the processor faces'
    cells and interfaceBouCoeffs (patch after patch) and the communicator
    that serves them."""

    def __init__(self, face_cells, coeffs, comm: ProcessorComm):
        self.face_cells = np.ascontiguousarray(face_cells, dtype=np.int32)
        self.coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        if len(self.face_cells) != len(self.coeffs):
            raise ValueError("face_cells and coeffs differ in length")
        if comm.n_faces != len(self.face_cells):
            raise ValueError("the communicator's patches do not match the faces")
        self.comm = comm

    @classmethod
    def from_subdomain(cls, sub: Subdomain, group=None) -> "ProcessorInterfaces":
        fc, co = sub.interface_arrays()
        return cls(fc, co, ProcessorComm(sub.patches, group))

    @property
    def n_faces(self) -> int:
        return len(self.face_cells)

    def as_c(self):
        """(cf_interfaces, cf_comm) for cf_solve_decomposed."""
        i = _capi.cf_interfaces()
        i.n_faces = self.n_faces
        i.face_cells = self.face_cells.ctypes.data if self.n_faces else None
        i.coeffs = self.coeffs.ctypes.data if self.n_faces else None
        return i, self.comm.as_c()


def amul_decomposed(sub: Subdomain, x_local: np.ndarray, ghosts: np.ndarray) -> np.ndarray:
    """lduMatrix::Amul on one subdomain in numpy: the local product, then
    ``result[face_cells[f]] -= coeffs[f] * ghosts[f]`` in face order.  Host
    reference for tests of the decomposition and of the exchange."""
    y = sub.diag * x_local
    np.add.at(y, sub.upper_addr, sub.lower * x_local[sub.lower_addr])
    np.add.at(y, sub.lower_addr, sub.upper * x_local[sub.upper_addr])
    fc, co = sub.interface_arrays()
    np.subtract.at(y, fc, co * ghosts)
    return y
