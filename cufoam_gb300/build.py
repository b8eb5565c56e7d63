"""Build the library in-tree: nvcc, one -gencode for sm_103a, translation
units compiled in parallel, linked into ``cufoam_gb300/_build/libcufoam_gb300.so``
(a plain C-ABI shared library: no Python or torch symbols)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libcufoam_gb300.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)

SOURCES = ["capi.cu", "matrix.cu", "solve_fp64.cu", "solve_fast.cu", "mixed.cu", "adjoint.cu", "batched.cu",
           "noalloc.cu", "distributed.cu", "formats.cpp"]
HEADERS = ["internal.h", "device.cuh", "solver_common.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    # CUFOAM_NVCC_DEFINES: extra -D definitions for the kernel tuning
    # constants (CF_SELL_BATCH, CF_SPMV_MIN_BLOCKS, ...) when sweeping them
    extra = os.environ.get("CUFOAM_NVCC_DEFINES", "").split()
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I" + INCLUDE, "-I" + CSRC, "--expt-relaxed-constexpr"] + \
        [d for d in extra if d.startswith("-D")]


def _newest(paths: list[str]) -> float:
    return max(os.path.getmtime(p) for p in paths)


PLUGIN_DIR = os.path.join(HERE, "plugin")
PLUGIN_LIB = os.path.join(BUILD_DIR, "libcufoam_plugin_minifoam.so")


def build_plugin(force: bool = False) -> str:
    """The OpenFOAM plugin sources compiled against the minifoam stand-in,
    plus the harness that drives them (linked to the C-ABI library)."""
    srcs = [os.path.join(PLUGIN_DIR, "cuFoamGB300.C"),
            os.path.join(PLUGIN_DIR, "minifoam", "minifoam_harness.C")]
    deps = srcs + [os.path.join(PLUGIN_DIR, "cuFoamGB300.H"),
                   os.path.join(PLUGIN_DIR, "cuFoamGB300Comm.H"),
                   os.path.join(PLUGIN_DIR, "minifoam", "lduMatrix.H"),
                   os.path.join(INCLUDE, "cufoam_gb300.h"), LIB_PATH]
    if force or not os.path.exists(PLUGIN_LIB) or os.path.getmtime(PLUGIN_LIB) < _newest(deps):
        tmp = PLUGIN_LIB + f".tmp{os.getpid()}"
        cmd = ["g++", "-O2", "-std=c++14", "-shared", "-fPIC", "-Wall",
               "-I" + os.path.join(PLUGIN_DIR, "minifoam"), "-I" + INCLUDE] + srcs + \
              ["-L" + BUILD_DIR, "-lcufoam_gb300", "-Wl,-rpath,$ORIGIN", "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"plugin build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, PLUGIN_LIB)
    return PLUGIN_LIB


COMPAT_DIR = os.path.join(HERE, "compat")
GIS_LIB = os.path.join(BUILD_DIR, "libGIS.so")
GIS_HARNESS = os.path.join(BUILD_DIR, "libgis_harness.so")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def build_gis(force: bool = False) -> str:
    """libGIS.so: the reference solver library's gis.h interface on this
    library (compat/gis_compat.cu), plus the ctypes harness that drives it
    as the plugins do."""
    src = os.path.join(COMPAT_DIR, "gis_compat.cu")
    hdr = os.path.join(COMPAT_DIR, "SingleGPUCompat.h")
    deps = [src, hdr, os.path.join(CSRC, "internal.h"), os.path.join(INCLUDE, "cufoam_gb300.h"), LIB_PATH]
    if force or not os.path.exists(GIS_LIB) or os.path.getmtime(GIS_LIB) < _newest(deps):
        tmp = GIS_LIB + f".tmp{os.getpid()}"
        cmd = [nvcc()] + _flags() + ["-I" + COMPAT_DIR, "-shared", src, "-o", tmp,
                                     "-L" + BUILD_DIR, "-lcufoam_gb300", "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"libGIS build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, GIS_LIB)
    hsrc = os.path.join(COMPAT_DIR, "gis_harness.cpp")
    if force or not os.path.exists(GIS_HARNESS) or os.path.getmtime(GIS_HARNESS) < _newest([hsrc, hdr, GIS_LIB]):
        tmp = GIS_HARNESS + f".tmp{os.getpid()}"
        cu = cuda_home()
        cmd = ["g++", "-O2", "-std=c++14", "-shared", "-fPIC", "-Wall", "-I" + COMPAT_DIR,
               "-I" + os.path.join(cu, "include"), hsrc, "-L" + BUILD_DIR, "-lGIS",
               "-L" + os.path.join(cu, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN", "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"gis harness build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, GIS_HARNESS)
    return GIS_LIB


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "cufoam_gb300.h")]
    hdr_time = _newest(hdrs)
    objs = []
    jobs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        op = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(op)
        if force or not os.path.exists(op) or os.path.getmtime(op) < max(os.path.getmtime(sp), hdr_time):
            jobs.append((sp, op))

    def compile_one(job):
        sp, op = job
        tmp = op + f".tmp{os.getpid()}"
        cmd = [nvcc()] + _flags() + ["-c", sp, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {sp}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        os.replace(tmp, op)

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, jobs))
    if jobs or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < _newest(objs):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    build_plugin(force)
    build_gis(force)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
