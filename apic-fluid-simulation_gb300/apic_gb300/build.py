"""Compile the sm_103a CUDA library (libapic_gpu.so) in-tree.

The translation units compile in parallel with one ``-gencode`` each and link
into ``apic-fluid-simulation_gb300/lib/libapic_gpu.so`` with the CUDA runtime
linked statically.  ``-fmad=false`` keeps every multiply-add exactly as
written (the kernels use ``__fmaf_rn`` where the reference calls ``mul_add``).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libapic_gpu.so")

CUDA_SOURCES = ["sort.cu", "particles.cu", "grid.cu", "vcycle.cu", "vcycle_dsm.cu", "solver.cu", "batch.cu",
                "runtime.cu", "noalloc.cu", "serve.cu", "render.cu"]
CXX_SOURCES = ["scene.cpp"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math", "--expt-relaxed-constexpr",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


CHECKED_BUILD_DIR = os.path.join(PKG_ROOT, "_build_checked")
CHECKED_LIB_PATH = os.path.join(LIB_DIR, "libapic_gpu_checked.so")


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False, checked: bool = False) -> str:
    """Build libapic_gpu.so if any source changed; return its path.

    checked: build libapic_gpu_checked.so instead, with -DAPIC_BOUNDS_CHECK
    (data-dependent indices tested before use; an update that met one
    outside its buffer fails with APIC_ERR_CUDA)."""
    build_dir = CHECKED_BUILD_DIR if checked else BUILD_DIR
    lib_path = CHECKED_LIB_PATH if checked else LIB_PATH
    extra = ["-DAPIC_BOUNDS_CHECK"] if checked else []
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(PKG_ROOT), "include", "apic_gpu.h"))
    jobs = []
    objs = []
    for src in CUDA_SOURCES + CXX_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(build_dir, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            if src.endswith(".cu"):
                cmd = [nvcc] + NVCC_FLAGS + extra + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", path, "-o", obj]
            else:
                cmd = ["g++"] + CXX_FLAGS + ["-c", path, "-o", obj]
            jobs.append(cmd)
    outs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for o in outs:
            if o.strip():
                sys.stderr.write(o)
    if force or jobs or _stale(lib_path, objs):
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", lib_path] + objs + ["-lpthread", "-ldl", "-lrt"])
    return lib_path


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv,
                checked="--checked" in sys.argv))
