"""Builds the in-tree shared library ``fmca_gb300/libfmca_gb300.so``.

Host sources are compiled with g++ (``-ffp-contract=off`` keeps the plan's
floating-point decisions identical on x86-64 and aarch64), CUDA sources with
nvcc for sm_103a only; everything is linked by nvcc into one shared library
whose exported C symbols are declared in ``include/fmca_gb300.h``.  Object
files go to ``fmca_gb300/_build/``; compilations run in parallel and are
skipped when the object is newer than its sources.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "libfmca_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall",
             "-Wno-unused-function"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
              "-Xptxas", "-O3"] + ARCH

HOST_SOURCES = ["h2_plan.cpp", "plan_io.cpp", "near_pack.cpp", "c_api.cpp"]
CUDA_SOURCES = ["h2_gpu.cu", "h2_static_scratch.cu", "h2_tree_gpu.cu", "h2_umma_persistent.cu",
                "h2_assembled.cu", "h2_far_kron.cu"]
HEADERS = ["h2_plan.h", "plan_io.h", "near_pack.h", "h2_gpu.h", "compensated_sum.h", "h2_gpu_kernels.cuh", "h2_tc_kernels.cuh", "h2_umma_kernels.cuh", "umma.cuh",
           "h2_umma_persistent.cuh", "h2_umma_persistent.h",
           "h2_adjoint_kernels.cuh", "c_api_internal.h", "h2_assembled.h",
           "h2_assembled_kernels.cuh", "h2_far_kron.h", "h2_far_kron.cuh"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fmca_gb300")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def build(verbose: bool = False) -> str:
    """Compiles and links the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(), "include")
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "fmca_gb300.h")]
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not _newer(o, [s] + hdrs + [__file__]):
            jobs.append(["g++"] + CXX_FLAGS + ["-I", cuda_inc, "-I", INCLUDE, "-c", s, "-o", o])
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not _newer(o, [s] + hdrs + [__file__]):
            jobs.append([nvcc] + NVCC_FLAGS + ["-I", INCLUDE, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if jobs or not _newer(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc, "-shared"] + ARCH + objs + ["-o", tmp, "-lcudart"])
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
