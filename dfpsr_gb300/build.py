"""Builds the in-tree CUDA library of the DFPSR triangle path (libdsrg.so) for sm_103a.

Device code is compiled with -fmad=false and host code with -ffp-contract=off: the
renderer's results are defined by binary32 operations in a fixed order, and a fused
multiply-add anywhere would change them.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdsrg.so")
SOURCES = ["dsrg_kernels.cu", "dsrg_api.cu", "dsrg_noalloc.cu", "dsrg_pipeline.cu", "dsrg_batch.cu", "dsrg_diff.cu", "dsrg_light.cu", "dsrg_sort.cu", "dsrg_occlusion.cu", "dsrg_texture.cu", "dsrg_overlay.cu", "dsrg_dense.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def headers():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    out.append(os.path.join(os.path.dirname(HERE), "include", "dsrg.h"))
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = headers()
    objs = []
    jobs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [path] + hdrs):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", path, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as pool:
        for f in [pool.submit(run, j) for j in jobs]:
            f.result()
    if force or jobs or _stale(LIB, objs):
        run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread", "-Xlinker", "--no-undefined"])
    return LIB


HOSTCHECK_LIB = os.path.join(HERE, "libdsrg_hostcheck.so")


def build_hostcheck(force: bool = False) -> str:
    """Host build of the kernels' exact arithmetic, for CPU-side checks."""
    src = os.path.join(CSRC, "dsrg_hostcheck.cpp")
    if force or _stale(HOSTCHECK_LIB, [src] + headers()):
        cxx = os.environ.get("CXX", "g++")
        subprocess.check_call([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", HOSTCHECK_LIB])
    return HOSTCHECK_LIB


SHIM_DIR = os.path.join(HERE, "dsr")


def build_shim(reference_source: str, out_dir: str = BUILD) -> str:
    """Compiles the dsr::gpu shim (dsr/dsr_gpu.cpp) against the reference's headers, as a program
    using the reference links it: reference_source is the reference's Source/ directory.  Returns
    the object file; link it with the reference's library and libdsrg.so."""
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(SHIM_DIR, "dsr_gpu.cpp")
    obj = os.path.join(out_dir, "dsr_gpu.o")
    deps = [src, os.path.join(SHIM_DIR, "dsr_gpu.h"), os.path.join(os.path.dirname(HERE), "include", "dsrg.h")]
    if _stale(obj, deps):
        cxx = os.environ.get("CXX", "g++")
        # the reference's own release flags (C++14, NDEBUG); no contraction, like the rest of the path
        subprocess.check_call([cxx, "-std=c++14", "-O2", "-DNDEBUG", "-ffp-contract=off", "-fPIC", "-I", reference_source,
                               "-I", os.path.join(os.path.dirname(HERE), "include"), "-c", src, "-o", obj])
    return obj


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    build_hostcheck(force="--force" in sys.argv)
