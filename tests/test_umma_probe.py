"""The tcgen05 operand layouts that the tensor-core kernel sums rely on:
A in tensor memory (row m in lane m, two K elements per 32-bit column), B in
shared memory as K-major core matrices without swizzle, D in tensor memory.
One exact 128 x 32 x 16 product of small integers, built from
tests/cuda/umma_layout_probe.cu with the library's own PTX wrappers."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np
import pytest

from fmca_gb300 import build as fbuild

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _probe_lib(tmp):
    src = os.path.join(ROOT, "tests", "cuda", "umma_layout_probe.cu")
    out = os.path.join(tmp, "libumma_probe.so")
    cmd = [fbuild._nvcc(), "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
           *fbuild.ARCH, "-I", os.path.join(ROOT, "fmca_gb300", "csrc"), src, "-o", out]
    subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    lib = ctypes.CDLL(out)
    lib.umma_probe.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_int]
    lib.umma_probe.restype = ctypes.c_int
    return lib


def test_tcgen05_operand_layouts(cuda_device, tmp_path):
    lib = _probe_lib(str(tmp_path))
    m = np.arange(128)[:, None]
    k = np.arange(16)[None, :]
    A = ((m * 7 + k * 3) % 11 - 5).astype(np.float64)
    kk = np.arange(16)[:, None]
    n = np.arange(32)[None, :]
    B = ((kk * 5 + n) % 7 - 3).astype(np.float64)
    for twice in (0, 1):
        out = np.zeros((128, 32), np.float32)
        rc = lib.umma_probe(out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), twice)
        assert rc == 0
        assert np.array_equal(out.astype(np.float64), (1 + twice) * (A @ B))
