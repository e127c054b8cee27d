"""Builds the native libraries of the package in-tree (``simplefem_gb300/_lib``).

* ``libfeec_gpu.so``      — sm_103a kernels + the C ABI of ``include/feec_gpu.h``
* ``libfeec_dropin.so``   — the reference's C++ solver entry points over that ABI
* ``libfeec_workload.so`` — host-side synthetic FEM workloads (lattice assembler)

Translation units are compiled in parallel; nothing is rebuilt if the outputs are
newer than every source. ``python -m simplefem_gb300.build`` runs it by hand.
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
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-O3",
              "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-I" + INCLUDE, "-I" + CSRC]

GPU_SOURCES = ["kernels_krylov.cu", "kernels_eisenstat.cu", "kernels_setup.cu", "capi.cu", "coloring.cpp", "noalloc.cu", "kernels_batched.cu", "batched.cu", "kernels_cluster.cu", "kernels_cluster_batched.cu", "server.cu", "selftest.cu", "csr_algebra.cu", "kernels_krylov_more.cu", "hodge.cu", "kernels_small.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build simplefem_gb300")


def _newer(target: str, sources) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr.strip():
        print(res.stderr, flush=True)
    return res


def lib_path(name: str) -> str:
    return os.path.join(LIBDIR, name)


def build(verbose: bool = False, force: bool = False) -> dict:
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    cc = nvcc()
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(cc))), "include")
    cxx = CXX_FLAGS + ["-I" + cuda_inc]
    out = {}

    # 1) GPU library
    gpu_so = lib_path("libfeec_gpu.so")
    srcs = [os.path.join(CSRC, s) for s in GPU_SOURCES]
    if force or not _newer(gpu_so, srcs + headers):
        jobs = []
        objs = []
        for s in srcs:
            obj = os.path.join(OBJDIR, os.path.basename(s) + ".o")
            objs.append(obj)
            if s.endswith(".cu"):
                cmd = [cc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", obj]
            else:
                cmd = ["g++", *cxx, "-c", s, "-o", obj]
            jobs.append(cmd)
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
        _run([cc, *ARCH, "-shared", "-o", gpu_so, *objs, "-lpthread"], verbose)
    out["gpu"] = gpu_so

    # 2) drop-in shim with the reference's mangled names, linked to the GPU library
    shim_so = lib_path("libfeec_dropin.so")
    shim_src = os.path.join(CSRC, "dropin_shim.cpp")
    if force or not _newer(shim_so, [shim_src, gpu_so] + headers):
        _run(["g++", *CXX_FLAGS, "-shared", shim_src, "-o", shim_so, "-L" + LIBDIR, "-lfeec_gpu",
              "-Wl,-rpath,$ORIGIN"], verbose)
    out["dropin"] = shim_so

    # 3) workload assembler (host only)
    wl_so = lib_path("libfeec_workload.so")
    wl_src = os.path.join(CSRC, "lattice_fem.cpp")
    if force or not _newer(wl_so, [wl_src]):
        _run(["g++", *CXX_FLAGS, "-fopenmp", "-shared", wl_src, "-o", wl_so], verbose)
    out["workload"] = wl_so
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
