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


C_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "fmca_gb300.h"

int main(void) {
  enum { N = 3000 };
  double* P = (double*)malloc(sizeof(double) * 3 * N);
  unsigned s = 1u;
  for (int i = 0; i < 3 * N; ++i) {
    s = s * 1664525u + 1013904223u;
    P[i] = (s >> 8) / 16777216.0;
  }
  fmca_plan* tp = NULL;
  fmca_plan* td = NULL;
  if (fmca_plan_create(P, 3, N, NULL, N, 3, 0.8, 64, &tp) != FMCA_OK) return 1;
  if (fmca_plan_create_ex(P, 3, N, NULL, N, FMCA_INTERP_TOTAL_DEGREE, 4, 0.8, 0, &td) != FMCA_OK)
    return 2;
  int64_t a[FMCA_INFO_COUNT], b[FMCA_INFO_COUNT];
  double st[6], nodes[3 * 35];
  if (fmca_plan_info(tp, a) != FMCA_OK || fmca_plan_info(td, b) != FMCA_OK) return 3;
  if (fmca_plan_statistics(td, st) != FMCA_OK) return 4;
  if (fmca_plan_interpolator(td, nodes, NULL) != FMCA_OK) return 5;
  printf("%lld %lld %lld %lld %.17g %.17g\n", (long long)a[FMCA_INFO_Q],
         (long long)b[FMCA_INFO_Q], (long long)a[FMCA_INFO_INTERPOLATOR],
         (long long)b[FMCA_INFO_INTERPOLATOR], st[0], nodes[0]);
  fmca_plan_destroy(tp);
  fmca_plan_destroy(td);
  free(P);
  return 0;
}
"""


def test_header_compiles_as_c_and_links(tmp_path):
    """A plain C99 program against include/fmca_gb300.h and the library, as a
    non-Python binding would use them (plan calls only, no GPU)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    _lib.load()
    src = tmp_path / "prog.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "prog"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", libdir,
                    "-lfmca_gb300", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out[:4] == ["64", "35", "0", "1"]
    assert float(out[4]) == 3000.0
    P = np.random.default_rng(0).random((3, 10))  # any plan: the nodes do not depend on points
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 4, 0.8, interpolator="total_degree")
    assert float(out[5]) == H.interpolation_nodes()[0][0, 0]


def test_tune_indices_match_the_binding():
    # the FMCA_TUNE_* indices of the header and the binding's key order
    txt = open(os.path.join(ROOT, "include", "fmca_gb300.h")).read()
    idx = {m.group(1).lower(): int(m.group(2))
           for m in re.finditer(r"\bFMCA_TUNE_([A-Z0-9_]+)\s*=\s*(\d+)", txt)}
    count = idx.pop("count")
    assert count == len(_lib.TUNE_KEYS) == len(idx)
    for key, i in idx.items():
        assert _lib.TUNE_KEYS[i] == {"us": "tune_us"}.get(key, key), key


def test_near_packed_argument_checks():
    lib = _lib.load()
    ng, ni = C.c_int64(0), C.c_int64(0)
    assert lib.fmca_plan_near_packed(None, C.byref(ng), C.byref(ni), None, None) == 1
    P = np.random.default_rng(16).random((2, 20000))
    H = H2Matrix(CovarianceKernel("MATERN32", 0.3), P, P, 3, 0.8)
    assert lib.fmca_plan_near_packed(H.handle, None, C.byref(ni), None, None) == 1
    assert lib.fmca_plan_near_packed(H.handle, C.byref(ng), C.byref(ni), None, None) == 0
    assert ng.value > 0 and ni.value > 0
    # arrays shorter than the counts are refused
    g = np.zeros((ng.value, 5), dtype=np.uint32)
    v = np.zeros((ni.value, 3), dtype=np.uint32)
    short = C.c_int64(ng.value - 1)
    assert lib.fmca_plan_near_packed(
        H.handle, C.byref(short), C.byref(ni), g.ctypes.data_as(C.POINTER(C.c_uint32)),
        v.ctypes.data_as(C.POINTER(C.c_uint32))) == 1
    groups, ivl = H.near_packed()
    assert groups.shape == (ng.value, 5) and ivl.shape == (ni.value, 3)
