"""The reference's matrix / vector file formats (gis/SparseSystem/SparseCPU.h)
read and written by the library (host code, no GPU): every fixture under
tests/golden/formats/ must read exactly as the reference's own readers read
it (expected arrays in formats_expected.npz, made by gen_formats.py), the
files our writers produce must be byte-identical to the reference's, and
round trips must be exact."""
import os

import numpy as np
import pytest

import cufoam_gb300 as cf
from cufoam_gb300._capi import CufoamError

HERE = os.path.dirname(os.path.abspath(__file__))
FMT = os.path.join(HERE, "golden", "formats")
EXP = np.load(os.path.join(HERE, "golden", "formats_expected.npz"))
NAMES = [str(n) for n in EXP["__names__"]]


@pytest.mark.parametrize("name", [n for n in NAMES if not n.startswith("vec")])
def test_matrix_file_reads_as_the_reference_reads_it(name):
    path = os.path.join(FMT, name)
    if not EXP[f"{name}/ok"][0]:
        with pytest.raises(CufoamError):
            cf.read_csr(path)
        return
    rows, cols, ro, ci, va = cf.read_csr(path)
    assert [rows, cols, va.shape[0]] == EXP[f"{name}/shape"].tolist()
    assert np.array_equal(ro, EXP[f"{name}/row_offsets"])
    assert np.array_equal(ci, EXP[f"{name}/cols"])
    assert va.tobytes() == EXP[f"{name}/vals"].tobytes()


@pytest.mark.parametrize("name", [n for n in NAMES if n.startswith("vec")])
def test_vector_file_reads_as_the_reference_reads_it(name):
    v = cf.read_vector(os.path.join(FMT, name))
    assert v.tobytes() == EXP[f"{name}/values"].tobytes()


def test_writers_match_the_reference_bytes(tmp_path):
    ro, ci, va = EXP["csr_in/row_offsets"], EXP["csr_in/cols"], EXP["csr_in/vals"]
    p = str(tmp_path / "a.bin")
    cf.save_csr(p, 5, 5, ro, ci, va)
    assert open(p, "rb").read() == EXP["saved_csr"].tobytes()
    q = str(tmp_path / "v.bin")
    cf.save_vector(q, EXP["vec_in"])
    assert open(q, "rb").read() == EXP["saved_vec"].tobytes()


def test_round_trips_and_symmetric_mirror(tmp_path):
    import oracle as O
    A = O.ldu2csr(O.grid_lognormal(6, 5, 4, 2))
    p = str(tmp_path / "m.csr")
    cf.save_csr(p, A.n, A.n, A.row_offsets, A.cols, A.vals)
    r, c, ro, ci, va = cf.read_csr(p)
    assert (r, c) == (A.n, A.n)
    assert np.array_equal(ro, A.row_offsets) and np.array_equal(ci, A.cols)
    assert va.tobytes() == A.vals.tobytes()
    # the symmetric fixture expands to a symmetric matrix with the stored triangle
    r, c, ro, ci, va = cf.read_csr(os.path.join(FMT, "rsa.rb"))
    D = np.zeros((r, c))
    for i in range(r):
        D[i, ci[ro[i]:ro[i + 1]]] = va[ro[i]:ro[i + 1]]
    assert np.array_equal(D, D.T)
    r, c, ro, ci, va = cf.read_csr(os.path.join(FMT, "rza.rb"))
    K = np.zeros((r, c))
    for i in range(r):
        K[i, ci[ro[i]:ro[i + 1]]] = va[ro[i]:ro[i + 1]]
    assert np.array_equal(K, -K.T)
    v = np.linspace(-1, 1, 33)
    q = str(tmp_path / "x.vec")
    cf.save_vector(q, v)
    assert cf.read_vector(q).tobytes() == v.tobytes()


def test_bad_files_are_errors(tmp_path):
    with pytest.raises(CufoamError):
        cf.read_csr(str(tmp_path / "missing.rb"))
    bad = tmp_path / "short.bin"
    bad.write_bytes(np.array([10, 10, 50], np.int32).tobytes() + b"\0" * 16)
    with pytest.raises(CufoamError):
        cf.read_csr(str(bad))
    t = tmp_path / "trunc.rb"
    t.write_text(open(os.path.join(FMT, "rua.rb")).read()[:-200])
    with pytest.raises(CufoamError):
        cf.read_csr(str(t))
    m = tmp_path / "c.mtx"
    m.write_text("%%MatrixMarket matrix array real general\n% a comment\n3 1\n1\n2\n")
    with pytest.raises(CufoamError):
        cf.read_vector(str(m))
    m.write_text("%%MatrixMarket matrix array real general\n% a comment\n3 1\n1\n2\n3.5\n")
    assert cf.read_vector(str(m)).tolist() == [1.0, 2.0, 3.5]
