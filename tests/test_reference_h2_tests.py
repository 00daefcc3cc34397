"""The reference's two H2 tests, restated with their parameters and the
total-degree interpolator they instantiate.

tests/test_H2Matrix.cpp:17-79: rows 2n, columns n (n = 10,000) uniform in
[-1, 1]^3, TotalDegreeInterpolator of degree 3, EXPONENTIAL l = 2, minimum
cluster size 0; the transfer identity is asserted < 1e-13 on both trees
(check_transfer_matrices, :46-49); for eta = 0.8, 0.4, 0.2 it prints
statistics() and the compression error of action() on 10 unit vectors
against exact kernel columns (:51-75).

tests/test_H2kernelActor.cpp:16-56: n = 10,000 uniform in [-1, 1]^2,
degree 4, EXPONENTIAL l = 1, the same eta sweep and unit-vector error.

The reference prints the errors; here they are bounded (with margin over
the oracle's values at seed 0) and must fall with eta. Points come from
numpy default_rng(0) instead of Eigen's unseeded Random()."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err
from fmca_gb300 import CovarianceKernel, H2Matrix

N = 10000
ETAS = (0.8, 0.4, 0.2)


@pytest.fixture(scope="module")
def h2matrix_case():
    rng = np.random.default_rng(0)
    Pr = rng.random((3, 2 * N)) * 2 - 1
    Pc = rng.random((3, N)) * 2 - 1
    X = np.zeros((N, 10))
    X[rng.integers(0, N, 10), np.arange(10)] = 1
    Yd = oracle.dense_matvec(0, 2.0, Pr, Pc, X)
    return Pr, Pc, X, Yd


@pytest.fixture(scope="module")
def actor_case():
    rng = np.random.default_rng(1)
    P = rng.random((2, N)) * 2 - 1
    X = np.zeros((N, 10))
    X[rng.integers(0, N, 10), np.arange(10)] = 1
    Yd = oracle.dense_matvec(0, 1.0, P, P, X)
    return P, X, Yd


def test_h2matrix_test(h2matrix_case):
    Pr, Pc, X, Yd = h2matrix_case
    errs = []
    for eta in ETAS:
        O = oracle.OraclePlan(Pr, Pc, p=3, eta=eta, min_leaf=0, interpolator="total_degree")
        assert O.check_transfer() < 1e-13
        H = H2Matrix(CovarianceKernel("EXPONENTIAL", 2.0), Pr, Pc, 3, eta,
                     interpolator="total_degree")
        assert np.array_equal(H.statistics(False).ravel(), O.statistics())
        Y, _ = O.action(0, 2.0, X)
        errs.append(rel_err(Y, Yd))
    assert errs[0] < 1e-3 and errs[0] > errs[1] > errs[2]
    assert errs[2] < 2e-5


def test_h2kernelactor_test(actor_case):
    P, X, Yd = actor_case
    errs = []
    for eta in ETAS:
        O = oracle.OraclePlan(P, None, p=4, eta=eta, min_leaf=0, interpolator="total_degree")
        Y, _ = O.action(0, 1.0, X)
        errs.append(rel_err(Y, Yd))
    assert errs[0] < 1e-4 and errs[0] > errs[1] > errs[2]
    assert errs[2] < 3e-6


@pytest.mark.gpu
@pytest.mark.parametrize("eta", [0.8, 0.2])
def test_h2matrix_test_on_gpu(cuda_device, h2matrix_case, eta):
    Pr, Pc, X, _ = h2matrix_case
    O = oracle.OraclePlan(Pr, Pc, p=3, eta=eta, min_leaf=0, interpolator="total_degree")
    Y_ref, _ = O.action(0, 2.0, X)
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 2.0), Pr, Pc, 3, eta,
                 precision="fp64", interpolator="total_degree")
    assert rel_err(H.action(X), Y_ref) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("eta", [0.8, 0.2])
def test_h2kernelactor_test_on_gpu(cuda_device, actor_case, eta):
    P, X, _ = actor_case
    O = oracle.OraclePlan(P, None, p=4, eta=eta, min_leaf=0, interpolator="total_degree")
    Y_ref, _ = O.action(0, 1.0, X)
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, 4, eta,
                 precision="fp64", interpolator="total_degree")
    assert rel_err(H.action(X), Y_ref) < 1e-12
