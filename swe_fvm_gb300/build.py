"""Builds the sm_103a shared library libswe_gb300.so in-tree.

Each .cu translation unit is compiled by nvcc in parallel, then linked with
nvcc into swe_fvm_gb300/_build/libswe_gb300.so.  Host code is compiled without
floating-point contraction (-ffp-contract=off) and device code without FMA
fusion (-fmad=false) unless SWE_GB300_FMAD=1, so the device arithmetic follows
the reference's operation order exactly.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libswe_gb300.so")
# checked build: every gathered index of the step kernels is range-checked on
# the device (a bad one sets an error bit instead of faulting)
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(BUILD_CHECKED, "libswe_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
SOURCES = ["swe_kernels.cu", "swe_precompute.cu", "swe_abi.cu", "swe_fp64_peak.cu", "swe_noalloc.cu", "swe_adjoint.cu",
           "swe_diagnostics.cu", "swe_layout.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def flags(checked: bool = False) -> list:
    fmad = os.environ.get("SWE_GB300_FMAD", "0") == "1"
    return ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O3",
            f"-fmad={'true' if fmad else 'false'}", "-I", INCLUDE, "-I", CSRC] + (["-DSWE_CHECKED"] if checked else [])


def _stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return any(os.path.getmtime(d) > t for d in deps) or os.environ.get("SWE_GB300_FMAD") is not None


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    lib, out_dir = (LIB_CHECKED, BUILD_CHECKED) if checked else (LIB, BUILD)
    if not force and not _stale(lib):
        return lib
    os.makedirs(out_dir, exist_ok=True)
    nv = nvcc()
    fl = flags(checked)

    def compile_one(src):
        obj = os.path.join(out_dir, src.replace(".cu", ".o"))
        cmd = [nv, *fl, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib + f".tmp{os.getpid()}"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
