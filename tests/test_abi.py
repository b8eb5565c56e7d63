"""CPU checks of the drop-in boundary: the C-ABI library builds for sm_103a,
loads, exports every function include/*.h declares, and the host-side
plugin surface (names, registration tables, controls) behaves like the
reference's.  No GPU compute happens here."""
import ctypes as C
import subprocess

import numpy as np
import pytest

import cufoam_gb300 as cf
from cufoam_gb300 import _capi
from conftest import HAVE_GPU


def test_library_exports_every_header_function():
    lib = _capi.load()
    declared = _capi.header_functions()
    assert "cf_solve" in declared and "cf_matrix_create_ldu" in declared
    out = subprocess.run(["nm", "-D", "--defined-only", _capi.lib_path()],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    for f in declared:
        assert hasattr(lib, f)


def test_library_has_no_torch_or_python_dependency():
    out = subprocess.run(["readelf", "-d", _capi.lib_path()], capture_output=True, text=True,
                         check=True).stdout
    assert "torch" not in out and "python" not in out.lower()


def test_library_is_built_for_sm_103a():
    out = subprocess.run(["readelf", "-S", _capi.lib_path()], capture_output=True, text=True,
                         check=True).stdout
    assert ".nv_fatbin" in out


def test_pure_host_entry_points():
    lib = _capi.load()
    assert lib.cf_abi_version() == 1
    assert lib.cf_status_string(0) == b"ok"
    assert lib.cf_status_string(2) == b"breakdown"
    k = C.c_int32(-1)
    for name, want in [("cuFoamCG", 0), ("BiCG", 1), ("cuFoamJacobi", 2), ("MR", 3),
                       ("cuFoamMRJacobi", 4), ("MRS", 5), ("cuFoamJMR", 6),
                       ("cuFoamRichardson", 7)]:
        assert lib.cf_solver_from_name(name.encode(), C.byref(k)) == 0
        assert k.value == want
    assert lib.cf_solver_from_name(b"cuFoamGAMG", C.byref(k)) == _capi.CF_BAD_INPUT
    c = _capi.cf_controls()
    lib.cf_controls_init(C.byref(c))
    assert c.tolerance == 1e-6 and c.max_iter == 1000 and c.bicg_int_bound == 1e-10
    assert c.power_max_steps == 30 and c.richardson_omega == 0.0 and c.use_graph == 1


@pytest.mark.skipif(HAVE_GPU, reason="checks the no-GPU error path")
def test_context_without_gpu_reports_no_device():
    lib = _capi.load()
    h = C.c_void_p()
    st = lib.cf_context_create(0, C.byref(h))
    assert st == _capi.CF_NO_DEVICE
    assert not h.value
    with pytest.raises(cf.CufoamError):
        cf.Context(0)


def test_null_arguments_are_rejected_without_a_device():
    lib = _capi.load()
    assert lib.cf_solve(None, 0, None, None, None, None) == _capi.CF_BAD_INPUT
    assert lib.cf_matrix_create_ldu(None, None, None) == _capi.CF_BAD_INPUT
    assert lib.cf_spmv(None, 0, None, None, 0, 0) == _capi.CF_BAD_INPUT


class _FakeMatrix:
    def __init__(self, sym):
        self._sym = sym

    def symmetric(self):
        return self._sym


def test_runtime_selection_tables():
    # CG and Richardson register only for symmetric matrices (and the
    # Jacobi-preconditioned CG, which has no reference counterpart)
    assert cf.solver_names(True) == sorted(["cuFoamBiCG", "cuFoamCG", "cuFoamJMR", "cuFoamJacobi",
                                            "cuFoamMR", "cuFoamMRJacobi", "cuFoamMRS",
                                            "cuFoamRichardson", "cuFoamPCG"])
    assert "cuFoamCG" not in cf.solver_names(False)
    assert "cuFoamRichardson" not in cf.solver_names(False)
    assert "cuFoamPCG" not in cf.solver_names(False)
    s = cf.New("p", _FakeMatrix(True), {"solver": "cuFoamCG", "tolerance": 1e-8})
    assert isinstance(s, cf.cuFoamCG) and s.type_name == "cuFoamCG"
    with pytest.raises(KeyError):
        cf.New("U", _FakeMatrix(False), {"solver": "cuFoamCG"})
    s = cf.New("U", _FakeMatrix(False), {"solver": "cuFoamBiCG"})
    assert s.kind == _capi.CF_BICG
    with pytest.raises(KeyError):
        cf.New("p", _FakeMatrix(True), {"solver": "PCG"})


def test_struct_layouts_match_header():
    # sizes computed by the C compiler for the header's structs
    src = r'''
#include "cufoam_gb300.h"
#include <stdio.h>
#include <stddef.h>
int main(void){printf("%zu %zu %zu %zu %zu\n", sizeof(cf_ldu_view), sizeof(cf_controls),
 sizeof(cf_perf), sizeof(cf_device_info), offsetof(cf_controls, time_limit_s)); return 0;}
'''
    import os
    import tempfile
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "s.c"), "w") as f:
        f.write(src)
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run(["gcc", "-I" + inc, os.path.join(d, "s.c"), "-o", os.path.join(d, "s")], check=True)
    sizes = [int(v) for v in subprocess.run([os.path.join(d, "s")], capture_output=True, text=True,
                                            check=True).stdout.split()]
    assert sizes == [C.sizeof(_capi.cf_ldu_view), C.sizeof(_capi.cf_controls),
                     C.sizeof(_capi.cf_perf), C.sizeof(_capi.cf_device_info),
                     _capi.cf_controls.time_limit_s.offset]


def test_header_enums_match_the_python_binding():
    """Every CF_ enum constant of include/cufoam_gb300.h has the value the
    ctypes binding uses (formats, memory kinds, statuses, solvers, ...)."""
    import os
    import re
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "cufoam_gb300.h")).read()
    found = {}
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    hdr = re.sub(r"//[^\n]*", "", hdr)
    for body in re.findall(r"enum\s*(?:\w+\s*)?\{([^}]*)\}", hdr):
        nxt = 0
        for item in body.split(","):
            item = item.strip()
            if not item:
                continue
            if "=" in item:
                name, val = (t.strip() for t in item.split("=", 1))
                nxt = int(val, 0)
            else:
                name = item
            found[name] = nxt
            nxt += 1
    assert found["CF_FORMAT_SELL_C8"] == 3 and found["CF_FORMAT_SELL_D16"] == 4
    checked = 0
    for name, val in found.items():
        if hasattr(_capi, name):
            assert getattr(_capi, name) == val, name
            checked += 1
    assert checked >= 10
