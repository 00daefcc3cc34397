"""The H2 part of the reference's Python module, name for name:
``import fmca_gb300.FMCA as FMCA`` in place of ``import FMCA``.

``H2Matrix(ker, Pr, Pc, p, eta)`` builds what pyH2Matrix builds
(py/FMCA.cpp:209-220): the total-degree interpolator of the module
(TotalDegreeInterpolator, py/FMCA.cpp:37-40), minimum cluster size 0 for both
trees (:216-217) and the pattern at ``eta``; the product is the FP64 GPU
product. Only what the module binds is exposed (:462-468): ``statistics()``
and ``action(rhs)`` (natural order in and out). ``CovarianceKernel`` takes
the module's constructors ``()``, ``(type)``, ``(type, l)``, ``(type, l,
c)`` and ``(type, l, c, nu)`` and binds ``kernelType()`` and ``eval(PR, PC)``
(:448-458). The wider interface (precisions, torch tensors, batching,
gradients) is ``fmca_gb300.H2Matrix``.
"""
from __future__ import annotations

import numpy as np

from .h2 import CovarianceKernel as _Kernel
from .h2 import H2Matrix as _H2Matrix

__all__ = ["CovarianceKernel", "H2Matrix"]


class CovarianceKernel(_Kernel):
    """CovarianceKernel(type="EXPONENTIAL", l=1, c=1, nu=1) of the module."""

    def __init__(self, ktype: str = "EXPONENTIAL", l: float = 1.0, c: float = 1.0,
                 nu: float = 1.0):
        super().__init__(ktype, l, c, nu)


class H2Matrix:
    """pyH2Matrix(ker, Pr, Pc, p, eta) on the GPU (FP64, total degree)."""

    def __init__(self, ker: _Kernel, Pr, Pc, p: int, eta: float):
        self._h = _H2Matrix(ker, Pr, Pc, p, eta, min_leaf=0, precision="fp64",
                            interpolator="total_degree")

    def statistics(self) -> np.ndarray:
        """(6, 1): rows, cols, low-rank blocks, dense blocks, nz per row, GB;
        printed like H2MatrixBase::statistics()."""
        return self._h.statistics(True)

    def action(self, rhs) -> np.ndarray:
        """y = K_H2 rhs, rhs: n_cols x R float64 (natural order)."""
        return self._h.action(np.asarray(rhs, dtype=np.float64))
