"""MultipoleFunctionEvaluator: kernel expansions evaluated at many points.

The reference's evaluator (FMCA/src/KernelInterpolation/
MultipoleFunctionEvaluator.h:17-62) builds an H2 matrix with the evaluation
points as rows and the data points as columns, total-degree interpolation,
eta = 0 and degree 3 by default; its test (tests/test_KernelInterpolation.cpp:
20-36) uses 10000 data and 2000 evaluation points in [0,1]^2, EXPONENTIAL
l = 1, eta = 0.5 and degree 10 (66 nodes per cluster, beyond the degree 7
of the tensor-product path).  Here the same configuration with random
coefficients (the samplet solver that computes them in the reference is out
of scope) against the FP64 oracle (1e-12) and the dense product (the
compression error, 1.4e-10 at degree 10)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err
from fmca_gb300 import CovarianceKernel, H2Matrix, MultipoleFunctionEvaluator

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(0)
    P = rng.random((2, 10000))
    Peval = rng.random((2, 2000))
    C = rng.standard_normal((10000, 2))
    return P, Peval, C


def test_reference_configuration(cuda_device, data):
    P, Peval, C = data
    kernel = CovarianceKernel("EXPONENTIAL", 1.0)
    mfe = MultipoleFunctionEvaluator(kernel, P, Peval, 0.5, 10)
    assert mfe.H.info["q"] == 66 and mfe.H.info["far_blocks"] > 0
    y = mfe.evaluate(P, Peval, C)
    assert y.shape == (2000, 2)
    O = oracle.OraclePlan(Peval, P, p=10, eta=0.5, min_leaf=0, interpolator="total_degree")
    y_ref, _ = O.action(0, 1.0, C)
    assert rel_err(y, y_ref) < 1e-12
    yd = oracle.dense_matvec(0, 1.0, Peval, P, C)
    assert rel_err(y, yd) < 1e-8
    # a vector of coefficients, as the reference's test passes
    assert rel_err(mfe.evaluate(P, Peval, C[:, 0]), y_ref[:, 0]) < 1e-12


def test_defaults_are_dense(cuda_device, data):
    # eta = 0 admits no far block: the evaluation is the dense sum
    P, Peval, C = data
    mfe = MultipoleFunctionEvaluator(CovarianceKernel("MATERN32", 0.3), P, Peval)
    assert mfe.eta == 0.0 and mfe.mpole_deg == 3 and mfe.H.info["far_blocks"] == 0
    yd = oracle.dense_matvec(1, 0.3, Peval, P, C)
    assert rel_err(mfe.evaluate(P, Peval, C), yd) < 1e-13


def test_moved_points_keep_the_structure(cuda_device, data):
    P, Peval, C = data
    kernel = CovarianceKernel("GAUSSIAN", 0.4)
    mfe = MultipoleFunctionEvaluator(kernel, P, Peval, 0.5, 6)
    P2 = P + 1e-3 * np.random.default_rng(1).standard_normal(P.shape)
    y = mfe.evaluate(P2, Peval, C)
    H = H2Matrix(kernel, Peval, P, 6, 0.5, precision="fp64", interpolator="total_degree")
    H.update_points(Peval, P2)
    assert rel_err(y, H.action(C)) < 1e-14
    yd = oracle.dense_matvec(3, 0.4, Peval, P2, C)
    assert rel_err(y, yd) < 1e-4
