"""Generates the file-format fixtures and their expected contents.

Writes small Rutherford-Boeing matrices (unsymmetric, rectangular,
symmetric, skew-symmetric, integer), a binary CSR file, Matrix Market and
binary vectors under tests/golden/formats/, reads every one of them with
the reference's own readers (CPU::SparseCSR::read, CPU::Vector::readMTX /
load from gis/SparseSystem/SparseCPU.h, built into oracle/_ref by
oracle/build.py) and stores what the reference read, plus the bytes of the
files the reference's writers produce, in tests/golden/formats_expected.npz.
Needs the reference sources; the committed outputs serve everywhere else.

    python tests/golden/gen_formats.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "formats")


def rb_text(title, key, mtype, nrow, ncol, colptr, rowind, vals, intvals=False):
    """A Rutherford-Boeing file: column pointers and row indices 1-based."""
    def block(xs, per, fmt):
        lines = []
        for i in range(0, len(xs), per):
            lines.append("".join(fmt(x) for x in xs[i:i + per]))
        return lines
    p = block([c + 1 for c in colptr], 10, lambda x: f"{x:8d}")
    r = block([i + 1 for i in rowind], 10, lambda x: f"{x:8d}")
    v = block(vals, 4, (lambda x: f"{int(x):20d}") if intvals else (lambda x: f"{x:20.12E}"))
    head = [f"{title:<72s}{key:<8s}",
            f"{len(p) + len(r) + len(v):14d}{len(p):14d}{len(r):14d}{len(v):14d}",
            f"{mtype:<3s}{'':11s}{nrow:14d}{ncol:14d}{len(vals):14d}{0:14d}",
            f"{'(10I8)':<16s}{'(10I8)':<16s}{'(4I20)' if intvals else '(4E20.12)':<20s}"]
    return "\n".join(head + p + r + v) + "\n"


def csc_from_dense(D, lower_only=False):
    colptr, rowind, vals = [0], [], []
    for j in range(D.shape[1]):
        for i in range(D.shape[0]):
            if (not lower_only or i >= j) and D[i, j] != 0:
                rowind.append(i)
                vals.append(D[i, j])
        colptr.append(len(rowind))
    return colptr, rowind, vals


def make_fixtures():
    os.makedirs(OUT, exist_ok=True)
    rng = np.random.default_rng(17)
    files = {}

    def sparse(m, n, dens):
        D = np.round(rng.standard_normal((m, n)) * 4, 3)
        D[rng.random((m, n)) > dens] = 0.0
        return D

    A = sparse(6, 6, 0.45)
    files["rua.rb"] = rb_text("unsymmetric 6x6", "RUA6", "rua", 6, 6, *csc_from_dense(A))
    R = sparse(4, 7, 0.5)
    files["rra.rb"] = rb_text("rectangular 4x7", "RRA47", "rra", 4, 7, *csc_from_dense(R))
    S = sparse(7, 7, 0.5)
    S = np.tril(S) + np.tril(S, -1).T + np.diag(np.arange(1.0, 8.0))
    files["rsa.rb"] = rb_text("symmetric 7x7", "RSA7", "rsa", 7, 7, *csc_from_dense(S, lower_only=True))
    K = sparse(5, 5, 0.6)
    K = np.tril(K, -1) - np.tril(K, -1).T
    files["rza.rb"] = rb_text("skew-symmetric 5x5", "RZA5", "rza", 5, 5, *csc_from_dense(K, lower_only=True))
    I = np.round(sparse(5, 5, 0.5))
    files["iua.rb"] = rb_text("integer 5x5", "IUA5", "iua", 5, 5, *csc_from_dense(I), intvals=True)
    files["cua.rb"] = rb_text("complex (rejected)", "CUA1", "cua", 1, 1, [0, 1], [0], [1.0])
    for name, text in files.items():
        with open(os.path.join(OUT, name), "w") as f:
            f.write(text)
    # a binary CSR file and vectors, written by this script byte by byte
    ro = np.array([0, 2, 3, 6, 6, 8], np.int32)
    ci = np.array([0, 4, 1, 0, 2, 3, 1, 4], np.int32)
    va = np.round(rng.standard_normal(8), 6)
    with open(os.path.join(OUT, "csr5.bin"), "wb") as f:
        f.write(np.array([5, 5, 8], np.int32).tobytes() + va.tobytes() + ro[:5].tobytes() + ci.tobytes())
    v = np.round(rng.standard_normal(9), 9)
    with open(os.path.join(OUT, "vec9.mtx"), "w") as f:
        f.write("%%MatrixMarket matrix array real general\n9 1\n" + "".join(f"{x:.17g}\n" for x in v))
    with open(os.path.join(OUT, "vec9.bin"), "wb") as f:
        f.write(np.array([9], np.int32).tobytes() + v.tobytes())
    return (ro, ci, va), v


def main():
    from oracle.build import build_ref_formats
    so = build_ref_formats()
    if so is None:
        raise SystemExit("the reference sources are needed to generate the expected outputs")
    (ro, ci, va), v = make_fixtures()
    L = C.CDLL(so)
    P = C.c_void_p
    L.ref_csr_read.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.ref_csr_take.argtypes = [P, P, P]
    L.ref_vec_read.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int)]
    L.ref_vec_take.argtypes = [P]
    L.ref_csr_save.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, P, P, P]
    L.ref_vec_save.argtypes = [C.c_char_p, C.c_int, P]
    out = {}
    names = []
    for name in sorted(os.listdir(OUT)):
        path = os.path.join(OUT, name).encode()
        if name.endswith(".rb") or name.endswith("csr5.bin"):
            r, c, z = C.c_int(), C.c_int(), C.c_int()
            rc = L.ref_csr_read(path, C.byref(r), C.byref(c), C.byref(z))
            names.append(name)
            out[f"{name}/ok"] = np.array([rc == 0])
            if rc == 0:
                a = np.zeros(r.value + 1, np.int32)
                b = np.zeros(max(z.value, 1), np.int32)
                d = np.zeros(max(z.value, 1))
                L.ref_csr_take(a.ctypes.data, b.ctypes.data, d.ctypes.data)
                out[f"{name}/shape"] = np.array([r.value, c.value, z.value], np.int64)
                out[f"{name}/row_offsets"], out[f"{name}/cols"], out[f"{name}/vals"] = a, b[:z.value], d[:z.value]
        elif name.startswith("vec"):
            n = C.c_int()
            rc = L.ref_vec_read(path, int(name.endswith(".mtx")), C.byref(n))
            names.append(name)
            out[f"{name}/ok"] = np.array([rc == 0])
            if rc == 0:
                x = np.zeros(max(n.value, 1))
                L.ref_vec_take(x.ctypes.data)
                out[f"{name}/values"] = x[:n.value]
    # bytes of the reference's writers
    tmp = os.path.join(OUT, "_ref_saved.bin")
    L.ref_csr_save(tmp.encode(), 5, 5, 8, np.ascontiguousarray(ro).ctypes.data,
                   np.ascontiguousarray(ci).ctypes.data, np.ascontiguousarray(va).ctypes.data)
    out["saved_csr"] = np.frombuffer(open(tmp, "rb").read(), np.uint8)
    L.ref_vec_save(tmp.encode(), v.shape[0], np.ascontiguousarray(v).ctypes.data)
    out["saved_vec"] = np.frombuffer(open(tmp, "rb").read(), np.uint8)
    os.remove(tmp)
    out["csr_in/row_offsets"], out["csr_in/cols"], out["csr_in/vals"], out["vec_in"] = ro, ci, va, v
    out["__names__"] = np.array(names)
    np.savez(os.path.join(HERE, "formats_expected.npz"), **out)
    print("wrote", len(names), "cases")


if __name__ == "__main__":
    main()
