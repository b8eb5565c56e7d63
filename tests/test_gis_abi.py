"""libGIS.so stand-in, CPU side: the library exports every gis.h function
(loading the harness resolves them), and -- where the reference sources are
present -- the harness compiled against the reference's own gis.h links to
this libGIS.so with no undefined symbol and sees the same container layouts
(SparseCSR / Vector field offsets) as the library's declarations."""
import os
import shutil
import subprocess

import pytest

from cufoam_gb300 import build as B
from cufoam_gb300.compat import GisHarness
from oracle.build import reference_root

# the reference's gis/ directory, where its sources are mounted (the oracle
# build recipe's location); the test skips elsewhere
REF_GIS = os.path.join(reference_root() or "", "gis")

EXPORTS = ["Transpose", "CG", "BiCG", "Richardson", "MR", "Jacobi", "MRJacobi", "JMR", "MRS",
           "NormFactor"]


@pytest.fixture(scope="module")
def built():
    B.build()
    return B.GIS_LIB


def test_libgis_exports(built):
    h = GisHarness()          # dlopen resolves every gis.h symbol the harness calls
    assert h.layout()[0] == 40 and h.layout()[6] == 16
    nm = shutil.which("nm")
    if nm:
        out = subprocess.run([nm, "-D", "-C", "--defined-only", built], capture_output=True,
                             text=True).stdout
        for name in EXPORTS:
            assert f" {name}(SingleGPU::" in out, name
        assert out.count(" BiCG(SingleGPU::") == 2


@pytest.mark.skipif(not reference_root() or not os.path.exists(os.path.join(REF_GIS, "gis.h")),
                    reason="reference sources not present")
def test_reference_header_links_to_libgis(built, tmp_path):
    out = tmp_path / "ref_harness.so"
    cmd = [B.nvcc(), "-x", "cu", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-DGH_REFERENCE_HEADER", "-I" + REF_GIS, os.path.join(B.COMPAT_DIR, "gis_harness.cpp"),
           "-o", str(out), "-L" + B.BUILD_DIR, "-lGIS", "-Xlinker", "--no-undefined",
           "-Xlinker", "-rpath," + B.BUILD_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    ref = GisHarness(str(out)).layout()
    ours = GisHarness().layout()
    assert ref == ours
