"""Special-function-unit rates behind the roofline of the kernel sums
(bench.py): ex2.approx runs at twice the rate of sqrt.approx, and a pair
(one sqrt, one ex2) costs the time of both on one pipe, i.e. 32 / 3 pairs
per clock per SM when ex2 gives 32 results per clock. Built from
tests/cuda/sfu_rate_probe.cu."""
from __future__ import annotations

import ctypes
import os
import subprocess

import pytest

from fmca_gb300 import build as fbuild

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sfu_rates_match_the_roofline_model(cuda_device, tmp_path):
    src = os.path.join(ROOT, "tests", "cuda", "sfu_rate_probe.cu")
    out = os.path.join(str(tmp_path), "libsfu_probe.so")
    subprocess.run([fbuild._nvcc(), "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                    *fbuild.ARCH, src, "-o", out], check=True, stdout=subprocess.PIPE,
                   stderr=subprocess.STDOUT)
    lib = ctypes.CDLL(out)
    ms = (ctypes.c_float * 3)()
    sms = ctypes.c_int(0)
    assert lib.sfu_probe(ms, ctypes.byref(sms)) == 0
    ex2, sqrt, pair = (2 ** 30 / ms[0], 2 ** 30 / ms[1], 2 ** 29 / ms[2])  # per ms
    per_sm_ns = [x / sms.value / 1e6 for x in (ex2, sqrt, pair)]
    print("sfu rates per SM per ns: ex2 %.2f, sqrt %.2f, pairs %.2f" % tuple(per_sm_ns))
    assert 1.7 < ex2 / sqrt < 2.3, (ex2, sqrt)
    model = 1.0 / (1.0 / ex2 + 1.0 / sqrt)
    assert 0.85 < pair / model < 1.1, (pair, model)
