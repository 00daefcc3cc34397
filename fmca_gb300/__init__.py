"""fmca_gb300 — GB300-native matrix-free H2-matrix kernel matvec.

A drop-in for the H2 hot path of FMCA (muchip/fmca): cluster trees and block
lists built on the host exactly like the reference, and the product computed
by hand-written sm_103a CUDA kernels behind the C ABI of
``include/fmca_gb300.h``.
"""
from ._lib import FmcaError, load  # noqa: F401
from .h2 import CovarianceKernel, H2Matrix, MultipoleFunctionEvaluator  # noqa: F401

__all__ = ["CovarianceKernel", "H2Matrix", "MultipoleFunctionEvaluator", "FmcaError", "load"]
