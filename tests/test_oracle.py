"""The oracle against the reference's own known-answer checks: the transfer
identity (compute_cluster_bases_impl.h:59-80, asserted < 1e-13 by
tests/test_H2Matrix.cpp:46-49) and the H2-vs-dense compression error the way
tests/test_H2Matrix.cpp:59-74 measures it."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err, sphere_cloud, uniform_cloud


@pytest.mark.parametrize("dim,deg,leaf", [(3, 3, 0), (3, 4, 96), (2, 5, 128), (1, 6, 0), (3, 1, 4)])
def test_transfer_identity(dim, deg, leaf):
    P = uniform_cloud(6000, dim, seed=dim * 10 + deg)
    O = oracle.OraclePlan(P, None, deg, 0.8, leaf)
    assert O.check_transfer() < 1e-13


def test_transfer_identity_unsymmetric_sphere():
    Pr = sphere_cloud(4000, seed=1)
    Pc = sphere_cloud(2500, seed=2)
    O = oracle.OraclePlan(Pr, Pc, 3, 0.8, 0)
    assert O.check_transfer() < 1e-13


def test_compression_error_unit_vectors():
    # test_H2Matrix.cpp: rows 2n, cols n, EXPONENTIAL l=2, 10 unit vectors
    rng = np.random.default_rng(0)
    n = 5000
    Pr = rng.random((3, 2 * n)) * 2 - 1
    Pc = rng.random((3, n)) * 2 - 1
    O = oracle.OraclePlan(Pr, Pc, 3, 0.8, 0)
    idx = rng.integers(0, n, 10)
    X = np.zeros((n, 10))
    X[idx, np.arange(10)] = 1
    Y, _ = O.action(0, 2.0, X)
    Yd = oracle.dense_matvec(0, 2.0, Pr, Pc, X)
    err = rel_err(Y, Yd)
    assert 0 < err < 1e-3


@pytest.mark.parametrize("ktype", list(range(10)))
def test_compression_error_all_kernels(ktype):
    P = uniform_cloud(4000, 3, seed=5)
    x = np.random.default_rng(5).standard_normal(4000)
    O = oracle.OraclePlan(P, None, 3, 0.8, 32)
    y, work = O.action(ktype, 0.5, x)
    yd = oracle.dense_matvec(ktype, 0.5, P, P, x)
    assert rel_err(y, yd) < 5e-4
    assert work[0] > 0 and work[1] > 0


def test_action_linear_and_scaled():
    P = uniform_cloud(3000, 3, seed=9)
    rng = np.random.default_rng(9)
    X = rng.standard_normal((3000, 3))
    O = oracle.OraclePlan(P, None, 2, 0.8, 16)
    Y, _ = O.action(1, 0.5, X, sigma2=2.5)
    y0, _ = O.action(1, 0.5, X[:, 0])
    assert rel_err(Y[:, 0], 2.5 * y0) < 1e-14
    yl, _ = O.action(1, 0.5, 2 * X[:, 0] - 3 * X[:, 1])
    Y1, _ = O.action(1, 0.5, X)
    assert rel_err(yl, 2 * Y1[:, 0] - 3 * Y1[:, 1]) < 1e-13


def test_kernel_formulas():
    # CovarianceKernel.h:64-113 at a few radii
    for r in (0.0, 0.3, 1.7):
        assert oracle.kernel(0, 0.5, r) == pytest.approx(np.exp(-r / 0.5), rel=1e-15)
        a = np.sqrt(3) / 0.5 * r
        assert oracle.kernel(1, 0.5, r) == pytest.approx((1 + a) * np.exp(-a), rel=1e-14)
        b = np.sqrt(5) / 0.5 * r
        assert oracle.kernel(2, 0.5, r) == pytest.approx((1 + b + b * b / 3) * np.exp(-b), rel=1e-14)
        assert oracle.kernel(3, 0.5, r) == pytest.approx(np.exp(-0.5 * r * r / 0.25), rel=1e-15)
    # BIHARMONIC2D (CovarianceKernel.h:56-59) and TPS2D (:117-118), zero at r = 0
    for r in (0.3, 1.0, 1.7):
        t = r / 0.5
        assert oracle.kernel(14, 0.5, r) == pytest.approx(np.log(t) * t * t, rel=1e-15)
        assert oracle.kernel(15, 0.5, r) == pytest.approx(r * r * np.log(r), rel=1e-15, abs=0)
    assert oracle.kernel(14, 0.5, 0.0) == 0.0 and oracle.kernel(14, 0.5, 1e-17) == 0.0
    assert oracle.kernel(15, 0.5, 0.0) == 0.0


@pytest.mark.parametrize("nparts", [2, 8])
def test_action_parts_reproduce_the_full_product(nparts):
    """oracle_action_part (the bounded samples of the timed CPU baseline):
    every part's rows equal the full product's rows bit for bit, and the
    parts' pair counts add up to the full product's (up to the blocks of the
    levels above the parts, which every part redoes)."""
    P = np.random.default_rng(3).random((3, 12000))
    X = np.random.default_rng(4).standard_normal((12000, 3))
    O = oracle.OraclePlan(P, None, 3, 0.8, 64)
    O.set_keep(True)
    Y, (dp, lp) = O.action(1, 0.5, X)
    perm = O.perm(0)
    Yp = np.full_like(Y, np.nan, order="F")
    seen = np.zeros(12000, dtype=bool)
    tot = np.zeros(2)
    for k in range(nparts):
        (b, n), work = O.action_part(1, 0.5, X, Yp, k, nparts)
        rows = perm[b:b + n]
        assert not seen[rows].any()
        seen[rows] = True
        assert np.array_equal(Yp[rows], Y[rows])
        tot += work
    assert seen.all()
    assert tot[0] >= dp and tot[1] >= lp
    assert tot[0] + tot[1] <= 1.02 * (dp + lp)
