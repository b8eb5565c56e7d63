"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/_build/liboracle.so`` -- the plain-C restatement (oracle.c),
  compiled with ``-ffp-contract=off`` so it gives the same bits on x86 and
  Arm, with OpenMP for the timed CPU baseline.
* ``oracle/_ref/libref_formats.so`` -- the reference's own matrix / vector
  file readers and writers (``gis/SparseSystem/SparseCPU.h``), compiled the
  same way, for the file-format golden fixtures.
* ``oracle/_ref/libref_ldu2csr.so`` -- the reference's own
  ``gis/ldu2csr.h`` compiled from its source file against the
  ``refstub/lduMatrix.H`` stand-in.  Built only where the reference sources
  are mounted; the committed golden fixtures carry its outputs elsewhere.
* ``oracle/_ref/ref_kernels.cubin`` (+ ``ref_kernels.names``) -- the
  reference's own device kernels (``gis/SparseSystem/kernels.h``,
  instantiated by ``refgpu/ref_kernels.cu``) compiled for sm_103a, with
  their entry names as ptxas lists them.  Built where the reference
  sources are mounted; the cubin is device code only, so the copy built
  here serves the GPU machine too.
* ``oracle/_build/librefgpu.so`` -- ``refgpu/ref_gpu.c``: the oracle
  backend that launches those kernels through the CUDA driver API.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "liboracle.so")
REF_LDU2CSR_SO = os.path.join(REF_DIR, "libref_ldu2csr.so")
REF_FORMATS_SO = os.path.join(REF_DIR, "libref_formats.so")
# Where this recipe reads the reference's sources: CUFOAM_REFERENCE_ROOT, or
# the read-only mount of the build machine.  Only the recipe names that
# mount; tests and tools ask reference_root(), which is None where neither
# exists (the GPU machine, which uses the outputs built here).
_DEFAULT_REFERENCE_MOUNT = "/root/reference"
REFERENCE_ROOT = os.environ.get("CUFOAM_REFERENCE_ROOT") or _DEFAULT_REFERENCE_MOUNT


def reference_root() -> str | None:
    """The reference source tree this recipe builds from, or None."""
    return REFERENCE_ROOT if os.path.isdir(REFERENCE_ROOT) else None


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "oracle.h")]
    if force or _stale(ORACLE_SO, srcs):
        tmp = ORACLE_SO + f".tmp{os.getpid()}"
        subprocess.check_call([
            "gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp",
            "-ffp-contract=off", "-Wall", srcs[0], "-o", tmp, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref_ldu2csr(force: bool = False) -> str | None:
    """Compile gis/ldu2csr.h from the reference sources, if they exist."""
    gis = os.path.join(REFERENCE_ROOT, "gis")
    hdr = os.path.join(gis, "ldu2csr.h")
    if not os.path.exists(hdr):
        return REF_LDU2CSR_SO if os.path.exists(REF_LDU2CSR_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    drv = os.path.join(HERE, "refstub", "ref_ldu2csr.cpp")
    stub = os.path.join(HERE, "refstub", "lduMatrix.H")
    if force or _stale(REF_LDU2CSR_SO, [drv, stub, hdr]):
        tmp = REF_LDU2CSR_SO + f".tmp{os.getpid()}"
        subprocess.check_call([
            "g++", "-O2", "-std=c++14", "-fPIC", "-shared",
            "-I" + gis, "-I" + os.path.join(HERE, "refstub"), drv, "-o", tmp])
        os.replace(tmp, REF_LDU2CSR_SO)
    return REF_LDU2CSR_SO


def build_ref_formats(force: bool = False) -> str | None:
    """Compile the reference's file readers / writers
    (gis/SparseSystem/SparseCPU.h), if the reference sources exist."""
    gis = os.path.join(REFERENCE_ROOT, "gis")
    hdr = os.path.join(gis, "SparseSystem", "SparseCPU.h")
    if not os.path.exists(hdr):
        return REF_FORMATS_SO if os.path.exists(REF_FORMATS_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    drv = os.path.join(HERE, "refstub", "ref_formats.cpp")
    if force or _stale(REF_FORMATS_SO, [drv, hdr]):
        tmp = REF_FORMATS_SO + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-I" + gis, drv, "-o", tmp])
        os.replace(tmp, REF_FORMATS_SO)
    return REF_FORMATS_SO


REF_CUBIN = os.path.join(REF_DIR, "ref_kernels.cubin")
REF_CUBIN_NAMES = os.path.join(REF_DIR, "ref_kernels.names")
REFGPU_SO = os.path.join(BUILD_DIR, "librefgpu.so")


def _entry_key(mangled: str) -> str:
    """The unqualified function name of an Itanium-mangled entry
    (_Z<len><name>...)."""
    i = 2
    j = i
    while j < len(mangled) and mangled[j].isdigit():
        j += 1
    n = int(mangled[i:j])
    return mangled[j:j + n]


def build_ref_kernels(force: bool = False) -> str | None:
    """Compile the reference's device kernels into a cubin, if the
    reference sources exist (otherwise keep a cubin built earlier)."""
    gis = os.path.join(REFERENCE_ROOT, "gis")
    hdr = os.path.join(gis, "SparseSystem", "kernels.h")
    if not os.path.exists(hdr):
        return REF_CUBIN if os.path.exists(REF_CUBIN) and os.path.exists(REF_CUBIN_NAMES) else None
    os.makedirs(REF_DIR, exist_ok=True)
    shim = os.path.join(HERE, "refgpu", "ref_kernels.cu")
    if force or _stale(REF_CUBIN, [shim, hdr]) or not os.path.exists(REF_CUBIN_NAMES):
        tmp = REF_CUBIN + f".tmp{os.getpid()}"
        # the reference's own flags (gis/CMakeLists.txt: -O3), one sm_103a target
        r = subprocess.run(["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                            "-I" + gis, "-Xptxas", "-v", shim, "-o", tmp],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {shim}:\n{r.stdout}\n{r.stderr}")
        names = []
        for line in (r.stdout + r.stderr).splitlines():
            if "Compiling entry function '" in line:
                mangled = line.split("'")[1]
                names.append(f"{_entry_key(mangled)} {mangled}")
        with open(REF_CUBIN_NAMES + ".tmp", "w") as f:
            f.write("\n".join(sorted(names)) + "\n")
        os.replace(REF_CUBIN_NAMES + ".tmp", REF_CUBIN_NAMES)
        os.replace(tmp, REF_CUBIN)
    return REF_CUBIN


def build_refgpu(force: bool = False) -> str:
    """The oracle backend that runs the reference's kernels (own source)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "refgpu", "ref_gpu.c")
    hdr = os.path.join(HERE, "oracle.h")
    if force or _stale(REFGPU_SO, [src, hdr]):
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(
            subprocess.check_output(["which", "nvcc"], text=True).strip()))), "include")
        tmp = REFGPU_SO + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
                               "-I" + cuda_inc, src, "-o", tmp, "-ldl", "-lm"])
        os.replace(tmp, REFGPU_SO)
    return REFGPU_SO


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_ref_ldu2csr(force)
    build_ref_formats(force)
    build_ref_kernels(force)
    build_refgpu(force)


if __name__ == "__main__":
    build_all(force=True)
    print(ORACLE_SO)
