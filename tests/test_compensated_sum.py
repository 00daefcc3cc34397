"""The compensated FP32 summation of the leaf gather
(fmca_gb300/csrc/compensated_sum.h, used by leafgather_kernel), compiled
for the host with g++ from the same header, in the kernel's loop shape:
plain FMA partial sums of kGatherBlock terms, each added into the total with
Kahan's compensation. Against a long-double reference the compensated sums
stay within a few kGatherBlock unit roundoffs of sum |terms| and beat the
plain sequential FP32 sum; exactly representable sums are exact."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "fmca_gb300", "csrc")

SRC = r"""
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "compensated_sum.h"
// reads the block size (0: kGatherBlock), q, then q pairs (v, s); prints
// plain, compensated, reference, abs-sum
int main() {
  int q, blk;
  if (scanf("%d %d", &blk, &q) != 2) return 1;
  if (blk <= 0) blk = fmca::kGatherBlock;
  float* v = new float[q];
  float* s = new float[q];
  for (int k = 0; k < q; ++k)
    if (scanf("%f %f", &v[k], &s[k]) != 2) return 1;
  float plain = 0.f;
  for (int k = 0; k < q; ++k) plain = std::fma(v[k], s[k], plain);
  float sum = 0.f, c = 0.f;
  for (int k0 = 0; k0 < q; k0 += blk) {
    const int k1 = q < k0 + blk ? q : k0 + blk;
    float part = 0.f;
    for (int k = k0; k < k1; ++k) part = std::fma(v[k], s[k], part);
    fmca::kahan_add(sum, c, part);
  }
  long double ref = 0, mag = 0;
  for (int k = 0; k < q; ++k) {
    ref += (long double)v[k] * (long double)s[k];
    mag += std::fabs((long double)v[k] * (long double)s[k]);
  }
  printf("%.9e %.9e %.21Le %.21Le\n", plain, sum, ref, mag);
  return 0;
}
"""


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("csum")
    src = d / "csum.cpp"
    src.write_text(SRC)
    exe = d / "csum"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, str(src),
                    "-o", str(exe)], check=True)
    return str(exe)


def run(prog, v, s, block=0):
    inp = f"{block} {len(v)}\n" + "\n".join(f"{a:.9e} {b:.9e}" for a, b in zip(v, s)) + "\n"
    out = subprocess.run([prog], input=inp, capture_output=True, text=True, check=True)
    plain, comp, ref, mag = (float(t) for t in out.stdout.split())
    return plain, comp, ref, mag


def test_compensated_gather_sum(prog):
    rng = np.random.default_rng(0)
    u = 2.0 ** -24
    worse_plain = 0
    for trial in range(40):
        q = int(rng.choice([10, 35, 64, 125, 216]))
        # the leaf gather's terms: basis values of mixed sign times
        # expansion coefficients of widely varying magnitude
        v = rng.standard_normal(q).astype(np.float32)
        s = (rng.standard_normal(q) * 10.0 ** rng.uniform(-3, 3, q)).astype(np.float32)
        plain, comp, ref, mag = run(prog, v, s)
        e_comp, e_plain = abs(comp - ref), abs(plain - ref)
        assert e_comp <= 4 * 8 * u * mag + 1e-30, (q, e_comp, mag)
        worse_plain += e_plain >= e_comp
    assert worse_plain >= 30  # the compensated sum is at least as close in most trials


def test_exact_sums_stay_exact(prog):
    v = np.ones(125, dtype=np.float32)
    s = np.arange(125, dtype=np.float32)
    plain, comp, ref, _ = run(prog, v, s)
    assert comp == ref == plain == 125 * 124 / 2
    # the Kahan step itself (blocks of one term): a large term followed by
    # many terms below its half ulp, which a plain FP32 sum drops
    s = np.array([2.0 ** 30] + [1.0] * 124, dtype=np.float32)
    plain, comp, ref, _ = run(prog, v, s, block=1)
    assert plain == 2.0 ** 30
    assert comp == float(np.float32(ref)) == 2.0 ** 30 + 128
