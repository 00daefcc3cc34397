"""Builds the oracle (test infrastructure): ``oracle/_build/libh2oracle.so``.

The FP64 restatement in ``h2_oracle.cpp`` is compiled with g++ -O3 -fopenmp
and -ffp-contract=off so that its tree and block lists round exactly like
the reference's (no fused multiply-adds on either x86-64 or aarch64).

The reference itself (muchip/fmca) is a header-only Eigen library and Eigen
is not available in this environment, so no ``oracle/_ref`` build exists.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libh2oracle.so")
SRC = os.path.join(HERE, "h2_oracle.cpp")


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(__file__)):
        return LIB
    cmd = ["g++", "-O3", "-fPIC", "-shared", "-std=c++17", "-fopenmp",
           "-ffp-contract=off", SRC, "-o", LIB + ".tmp"]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
