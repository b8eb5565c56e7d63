"""Generate the committed golden fixtures (run where the reference sources are
mounted; the fixtures then travel with the repository).

* ``ldu2csr_cases.npz`` -- LDU matrices with their lduAddressing and the CSR
  produced by the reference's own ``getSparseCSRMat`` (gis/ldu2csr.h:7-40),
  compiled from its source file by ``oracle/build.py`` (oracle/_ref).
* ``generator_checksums.json`` -- SHA-256 of the seeded synthetic inputs,
  pinning the generators to identical bytes on every host.

Usage:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def random_mesh(rng, n, n_faces, empty_tail=0):
    """Random upper-triangular face set over n cells (owner < neighbour),
    sorted by owner then neighbour; the last `empty_tail` cells get no
    faces at all."""
    m = n - empty_tail
    pairs = set()
    while len(pairs) < n_faces and m > 1:
        a, b = rng.integers(0, m, 2)
        if a != b:
            pairs.add((min(a, b), max(a, b)))
    pairs = sorted(pairs)
    la = np.array([p[0] for p in pairs], np.int32)
    ua = np.array([p[1] for p in pairs], np.int32)
    f = len(pairs)
    return O.LDU(n, rng.standard_normal(n) + 4.0, rng.standard_normal(f), rng.standard_normal(f),
                 la, ua)


def cases():
    rng = np.random.default_rng(20240521)
    out = {}
    out["c1_poisson_64x64"] = O.grid_const(64, 64, 1)
    out["lognormal_6x5x4"] = O.grid_lognormal(6, 5, 4, 11)
    cd, _ = O.grid_convdiff(5, 4, 3, 12)
    out["convdiff_5x4x3"] = cd
    out["random_n50_f120"] = random_mesh(rng, 50, 120)
    out["random_n200_f300_tail"] = random_mesh(rng, 200, 300, empty_tail=7)
    out["random_n17_f136_dense"] = random_mesh(rng, 17, 136)
    out["single_cell"] = O.LDU(1, np.array([2.5]), np.zeros(0), np.zeros(0),
                               np.zeros(0, np.int32), np.zeros(0, np.int32))
    out["two_cells_no_faces"] = O.LDU(2, np.array([1.0, -3.0]), np.zeros(0), np.zeros(0),
                                      np.zeros(0, np.int32), np.zeros(0, np.int32))
    perm = O.permutation(99, 4 * 4 * 3)
    out["permuted_lognormal_4x4x3"] = O.permute_ldu(O.grid_lognormal(4, 4, 3, 13), perm)
    return out


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def generator_inputs():
    """The synthetic inputs whose bytes are pinned across hosts."""
    g = {}
    g["c1_source_seed1"] = O.uniform(1, 4096)
    ln = O.grid_lognormal(8, 8, 8, 2)
    g["lognormal_8_seed2_diag"] = ln.diag
    g["lognormal_8_seed2_lower"] = ln.lower
    cd, _ = O.grid_convdiff(8, 8, 8, 4)
    g["convdiff_8_seed4_diag"] = cd.diag
    g["convdiff_8_seed4_lower"] = cd.lower
    g["convdiff_8_seed4_upper"] = cd.upper
    g["grf_12_seed5"] = O.grid_grf(12, 12, 12, 5, 8.0)
    g["perm_1000_seed7"] = O.permutation(7, 1000)
    g["normal_1000_seed9"] = O.normal(9, 1000)
    return g


def main():
    if not O.ref_ldu2csr_available():
        raise SystemExit("reference sources not mounted: cannot build oracle/_ref")
    arrays = {}
    names = []
    for name, L in cases().items():
        ls, lst, ost = L.addressing()
        ref = O.ref_ldu2csr(L)
        names.append(name)
        for k, v in (("n", np.array([L.n], np.int32)), ("diag", L.diag), ("lower", L.lower),
                     ("upper", L.upper), ("lower_addr", L.lower_addr),
                     ("upper_addr", L.upper_addr), ("losort", ls), ("losort_start", lst),
                     ("owner_start", ost), ("ref_row_offsets", ref.row_offsets),
                     ("ref_cols", ref.cols), ("ref_vals", ref.vals)):
            arrays[f"{name}/{k}"] = v
    arrays["__names__"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "ldu2csr_cases.npz"), **arrays)
    sums = {k: sha(v) for k, v in generator_inputs().items()}
    with open(os.path.join(HERE, "generator_checksums.json"), "w") as f:
        json.dump(sums, f, indent=1, sort_keys=True)
    print(f"wrote {len(names)} ldu2csr cases and {len(sums)} checksums")


if __name__ == "__main__":
    main()
