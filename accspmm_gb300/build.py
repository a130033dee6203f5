"""Builds libaccspmm.so and the `mma` command for sm_103a.

Every translation unit is compiled in parallel (nvcc for .cu, g++ for .cpp),
then linked into accspmm_gb300/libaccspmm.so (CUDA runtime linked statically)
and accspmm_gb300/bin/mma.  Objects go to accspmm_gb300/_build/.  A unit is
recompiled only when a source or header is newer than its object.

    python -m accspmm_gb300.build [--force]
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libaccspmm.so")
CLI = os.path.join(PKG, "bin", "mma")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# the product library
LIB_UNITS = ["host_formats.cpp", "metcf_io.cpp", "reorder.cpp", "permute.cu", "capi.cpp", "options.cpp",
             "device_prims.cu", "metcf_device.cu", "spmm.cu", "spmm_host.cpp", "spmm_batch.cu",
             "server.cpp", "gnn.cpp", "dense_gemm.cu"]
# the measurement build (libaccspmm_lab.so, -DACCSPMM_LAB): the same units plus
# the variant kernels kept for measurement (cp.async / bulk / tensor-map rings,
# lean, double-buffered, slice-major over staged B) and the gather floor
LAB_UNITS = LIB_UNITS + ["spmm_floor.cu", "spmm_pipe.cu", "spmm_bulk.cu", "spmm_lean.cu", "spmm_slice.cu"]
LAB_LIB = os.path.join(PKG, "libaccspmm_lab.so")


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h*")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit: str, force: bool, lab: bool = False) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, "lab" if lab else "", unit + ".o")
    if not force and not _stale(obj, [src] + _headers()):
        return obj
    cuda = cuda_home()
    inc = ["-I" + INCLUDE, "-I" + CSRC]
    defs = ["-DACCSPMM_LAB"] if lab else []
    if unit.endswith(".cu"):
        cmd = [os.path.join(cuda, "bin", "nvcc"), *ARCH, "-O3", "-std=c++17", "-lineinfo",
               "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", *defs, *inc, "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-Wno-unused-function",
               *defs, "-I" + os.path.join(cuda, "include"), *inc, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile of {unit} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _link(out: str, objs, force: bool) -> None:
    if not (force or _stale(out, objs)):
        return
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    lib64 = os.path.join(cuda, "lib64")
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", out, *objs, "-L" + lib64,
           "-Xlinker", "-rpath", "-Xlinker", lib64, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, lab: bool = True) -> str:
    """Builds libaccspmm.so and bin/mma; with `lab`, also the measurement build
    libaccspmm_lab.so (compiled in the same parallel pass)."""
    os.makedirs(os.path.join(BUILD, "lab"), exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    jobs = [(u, False) for u in LIB_UNITS + ["mma_main.cpp"]]
    if lab:
        jobs += [(u, True) for u in LAB_UNITS]
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(lambda j: _compile(j[0], force, j[1]), jobs))
    n = len(LIB_UNITS)
    lib_objs, cli_obj, lab_objs = objs[:n], objs[n], objs[n + 1:]
    cuda = cuda_home()
    _link(LIB, lib_objs, force)
    if lab:
        _link(LAB_LIB, lab_objs, force)
    objs = lib_objs + [cli_obj]
    if force or _stale(CLI, [objs[-1], LIB]):
        cmd = ["g++", "-o", CLI, objs[-1], "-L" + PKG, "-laccspmm",
               "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN/..",
               "-Wl,-rpath," + os.path.join(cuda, "lib64"), "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of mma failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB, "and", CLI)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
