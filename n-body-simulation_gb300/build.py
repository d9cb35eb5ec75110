"""Builds libnbody_cuda.so (CUDA kernels + C ABI, sm_103a) and the C++ host driver in-tree.

    python n-body-simulation_gb300/build.py            # everything
    python n-body-simulation_gb300/build.py cuda       # the CUDA library only

Outputs go to n-body-simulation_gb300/_build/. Translation units compile in parallel; no cmake.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter",
             "-ffp-contract=off", "-I", INCLUDE, "-I", HOST]

LIB_NAME = "libnbody_cuda.so"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_cuda(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(INCLUDE, "nbody.h")]
    objs = []
    jobs = []
    for src in sources:
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers) or ptxas_info:
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + [
                "-c", src, "-o", obj]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose or ptxas_info:
                sys.stdout.write(out)
    lib = os.path.join(OUT, LIB_NAME)
    if _stale(lib, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    return lib


def build_host(verbose: bool = False) -> str:
    """C++ host driver: the reference's CLI/CSV/ParaView surface over the C ABI."""
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if not srcs:
        return ""
    os.makedirs(OUT, exist_ok=True)
    headers = sorted(glob.glob(os.path.join(HOST, "*.hpp"))) + [os.path.join(INCLUDE, "nbody.h")]
    lib_host = os.path.join(OUT, "libnbody_host.so")
    exe = os.path.join(OUT, "nbody_sim")
    cuda_inc = os.path.join(cuda_home(), "include")
    cuda_lib = os.path.join(cuda_home(), "lib64")
    lib_srcs = [s for s in srcs if not s.endswith("main.cpp")]
    main_src = [s for s in srcs if s.endswith("main.cpp")]
    cxx = os.environ.get("CXX", "g++")
    if _stale(lib_host, lib_srcs + headers + [os.path.join(OUT, LIB_NAME)]):
        _run([cxx] + CXX_FLAGS + ["-I", cuda_inc, "-shared", "-o", lib_host] + lib_srcs +
             ["-L", OUT, "-lnbody_cuda", "-L", cuda_lib, "-lcudart", "-Wl,-rpath,$ORIGIN",
              "-Wl,-rpath," + cuda_lib])
    if main_src and _stale(exe, main_src + headers + [lib_host]):
        _run([cxx] + CXX_FLAGS + ["-I", cuda_inc, "-o", exe] + main_src +
             ["-L", OUT, "-lnbody_host", "-lnbody_cuda", "-L", cuda_lib, "-lcudart",
              "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + cuda_lib])
    return exe


def build_all(verbose: bool = False):
    lib = build_cuda(verbose)
    exe = build_host(verbose)
    return lib, exe


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what == "cuda":
        print(build_cuda(verbose=True))
    elif what == "ptxas":
        build_cuda(ptxas_info=True)
    else:
        print(build_all(verbose=True))
