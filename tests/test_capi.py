"""C ABI loading and host-side error handling (no GPU compute)."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

from fmca_gb300 import CovarianceKernel, FmcaError, H2Matrix, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "fmca_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fmca_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    syms = header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(_lib.EXPORTED) == syms


def test_version_and_kernel_names():
    lib = _lib.load()
    assert lib.fmca_version().startswith(b"fmca_gb300")
    t = C.c_int(-1)
    for i, name in enumerate(["EXPONENTIAL", "matern32", "Matern52", "GAUSSIAN"]):
        assert lib.fmca_kernel_type_from_name(name.encode(), C.byref(t)) == 0
        assert t.value == i
    assert lib.fmca_kernel_type_from_name(b"NOPE", C.byref(t)) == 2
    with pytest.raises(FmcaError):
        CovarianceKernel("NOT_A_KERNEL")


def test_plan_create_rejects_bad_arguments():
    lib = _lib.load()
    h = C.c_void_p()
    P = np.zeros((3, 10))
    dp = P.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.fmca_plan_create(None, 3, 10, None, 0, 3, 0.8, 0, C.byref(h)) == 1
    assert lib.fmca_plan_create(dp, 0, 10, None, 0, 3, 0.8, 0, C.byref(h)) == 1
    assert lib.fmca_plan_create(dp, 3, 0, None, 0, 3, 0.8, 0, C.byref(h)) == 1
    assert lib.fmca_plan_create(dp, 3, 10, None, 0, -1, 0.8, 0, C.byref(h)) == 1
    assert lib.fmca_plan_create(dp, 3, 10, None, 0, 3, float("nan"), 0, C.byref(h)) == 1
    P[0, 3] = np.inf
    assert lib.fmca_plan_create(dp, 3, 10, None, 0, 3, 0.8, 0, C.byref(h)) == 1
    assert b"non-finite" in lib.fmca_last_error()
    assert lib.fmca_plan_destroy(None) == 0


def test_matvec_argument_checks_without_gpu():
    lib = _lib.load()
    P = np.random.default_rng(0).random((3, 200))
    H = H2Matrix(CovarianceKernel("EXPONENTIAL"), P, P, 2, 0.8)
    k = CovarianceKernel("EXPONENTIAL").desc()
    dummy = C.c_void_p(16)
    # unknown precision / dtype / order / nrhs are rejected before any CUDA call
    assert lib.fmca_matvec(H.handle, C.byref(k), 7, 0, 0, 1, dummy, 1, 200, dummy, 1, 200,
                           None, 0, None) == 1
    assert lib.fmca_matvec(H.handle, C.byref(k), 0, 9, 0, 1, dummy, 1, 200, dummy, 1, 200,
                           None, 0, None) == 1
    assert lib.fmca_matvec(H.handle, C.byref(k), 0, 0, 5, 1, dummy, 1, 200, dummy, 1, 200,
                           None, 0, None) == 1
    assert lib.fmca_matvec(H.handle, C.byref(k), 0, 0, 0, 0, dummy, 1, 200, dummy, 1, 200,
                           None, 0, None) == 1
    bad = _lib.KernelDesc(0, -1.0, 1.0, 1.0, 1.0)
    assert lib.fmca_matvec(H.handle, C.byref(bad), 0, 0, 0, 1, dummy, 1, 200, dummy, 1, 200,
                           None, 0, None) == 1
    # dimension 4 builds a plan but the GPU path rejects it
    P4 = np.random.default_rng(0).random((4, 100))
    H4 = H2Matrix(CovarianceKernel("EXPONENTIAL"), P4, P4, 1, 0.8)
    n = C.c_size_t(0)
    assert lib.fmca_matvec_workspace_size(H4.handle, 0, 1, C.byref(n)) == 2


def test_workspace_size_grows_with_rhs():
    P = np.random.default_rng(0).random((3, 2000))
    H = H2Matrix(CovarianceKernel("EXPONENTIAL"), P, P, 3, 0.8)
    a, b = H.workspace_bytes(1, "mixed"), H.workspace_bytes(32, "mixed")
    assert 0 < a <= b < H.workspace_bytes(64, "mixed")
    assert H.workspace_bytes(1, "fp32") < H.workspace_bytes(32, "fp32")
    assert H.workspace_bytes(32, "fp64") > H.workspace_bytes(32, "fp32")
    assert b >= H.workspace_bytes(32, "fp32")
