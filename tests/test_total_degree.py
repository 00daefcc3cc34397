"""Total-degree interpolation (TotalDegreeInterpolator.h:26-47, the interpolator
of the reference's Python module, py/FMCA.cpp:37-40).

CPU: the plan's DeMarchi nodes (DeMarchiPoints.h:20-43) and inverse
Vandermonde matrix against the oracle's independent restatement (greedy
Gram-Schmidt selection and an LU inverse instead of Householder pivoting and
Gauss-Jordan), the reference's transfer identity (< 1e-13,
compute_cluster_bases_impl.h:66-76, run by tests/test_H2Matrix.cpp:46-49) on
the oracle, and the oracle's compression error against the dense product.
GPU: the matvec at every precision against the oracle on the same seeded
inputs, with the tolerances of tests/test_gpu_parity.py."""
from __future__ import annotations

import ctypes as C
from math import comb

import numpy as np
import pytest

import oracle
from conftest import rel_err, sphere_cloud, uniform_cloud
from fmca_gb300 import CovarianceKernel, H2Matrix, _lib

ERR = {v: k for k, v in _lib.STATUS_NAMES.items()}

CASES = [(1, 3), (2, 4), (2, 7), (3, 2), (3, 4), (3, 6), (2, 10), (2, 14), (1, 15)]


@pytest.mark.parametrize("dim,p", CASES)
def test_nodes_and_inverse_match_the_oracle(dim, p):
    P = uniform_cloud(2000, dim, seed=dim * 10 + p)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, p, 0.8,
                 interpolator="total_degree")
    O = oracle.OraclePlan(P, p=p, eta=0.8, interpolator="total_degree")
    q = comb(p + dim, dim)
    assert H.info["q"] == O.q == q
    assert H.info["interpolator"] == 1
    n1, i1 = H.interpolation_nodes()
    n2, i2 = O.interp()
    assert np.all((n1 >= 0) & (n1 <= 1))
    assert np.abs(n1 - n2).max() <= 1e-15
    assert np.abs(i1 - i2).max() <= 1e-12 * np.abs(i2).max()
    assert len(set(map(tuple, n1.T.round(15)))) == q  # distinct nodes
    # same tree and blocks as the oracle (the interpolator only sets q)
    assert H.info["far_blocks"] == O.n_far and H.info["near_blocks"] == O.n_near


def test_tensor_plan_reports_its_interpolator():
    P = uniform_cloud(500, 3, seed=3)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 3, 0.8)
    assert H.info["interpolator"] == 0 and H.info["q"] == 64
    nodes, invV = H.interpolation_nodes()
    assert invV is None
    assert np.allclose(np.sort(np.unique(nodes[0])),
                       np.sort(0.5 * (np.cos(np.pi * (np.arange(4) + 0.5) / 4) + 1)))


@pytest.mark.parametrize("dim,p", [(2, 5), (3, 4), (3, 6)])
def test_oracle_transfer_identity(dim, p):
    P = sphere_cloud(3000, seed=p) if dim == 3 else uniform_cloud(3000, dim, seed=p)
    O = oracle.OraclePlan(P, p=p, eta=0.8, min_leaf=32, interpolator="total_degree")
    assert O.check_transfer() < 1e-13


def test_oracle_compression_error_falls_with_degree():
    P = uniform_cloud(3000, 3, seed=5)
    x = np.random.default_rng(5).standard_normal((3000, 2))
    yd = oracle.dense_matvec(1, 0.5, P, P, x)
    errs = []
    for p in (2, 4, 6):
        O = oracle.OraclePlan(P, p=p, eta=0.8, min_leaf=32, interpolator="total_degree")
        assert O.n_far > 0
        errs.append(rel_err(O.action(1, 0.5, x)[0], yd))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 1e-5


def test_out_of_range_total_degree_is_refused():
    lib = _lib.load()
    P = np.asfortranarray(uniform_cloud(100, 4, seed=1))
    h = C.c_void_p()
    dp = P.ctypes.data_as(C.POINTER(C.c_double))
    st = lib.fmca_plan_create_ex(dp, 4, 100, None, 100, 1, 3, 0.8, 0, C.byref(h))
    assert st == ERR["FMCA_ERR_UNSUPPORTED"]
    P3 = np.asfortranarray(uniform_cloud(100, 3, seed=1))
    dp3 = P3.ctypes.data_as(C.POINTER(C.c_double))
    st = lib.fmca_plan_create_ex(dp3, 3, 100, None, 100, 1, 8, 0.8, 0, C.byref(h))
    assert st == ERR["FMCA_ERR_UNSUPPORTED"]  # 165 nodes
    P2 = np.asfortranarray(uniform_cloud(300, 2, seed=1))
    dp2 = P2.ctypes.data_as(C.POINTER(C.c_double))
    st = lib.fmca_plan_create_ex(dp2, 2, 300, None, 300, 1, 15, 0.8, 0, C.byref(h))
    assert st == ERR["FMCA_ERR_UNSUPPORTED"]  # 136 nodes
    assert lib.fmca_plan_create_ex(dp2, 2, 300, None, 300, 1, 14, 0.8, 0, C.byref(h)) == 0
    lib.fmca_plan_destroy(h)
    P1 = np.asfortranarray(uniform_cloud(300, 1, seed=1))
    dp1 = P1.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.fmca_plan_create_ex(dp1, 1, 300, None, 300, 1, 15, 0.8, 0, C.byref(h)) == 0
    lib.fmca_plan_destroy(h)
    st = lib.fmca_plan_create_ex(dp1, 1, 300, None, 300, 1, 16, 0.8, 0, C.byref(h))
    assert st == ERR["FMCA_ERR_UNSUPPORTED"]
    st = lib.fmca_plan_create_ex(dp3, 3, 100, None, 100, 7, 3, 0.8, 0, C.byref(h))
    assert st == ERR["FMCA_ERR_INVALID_ARGUMENT"]
    with pytest.raises(ValueError):
        H2Matrix(CovarianceKernel("MATERN32", 0.5), P3, P3, 3, 0.8, interpolator="sparse")


TOL = {"fp64": 1e-12, "fp32": 1e-5, "mixed": 1e-5}


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32", "mixed"])
@pytest.mark.parametrize("dim,p,kname", [(3, 4, "MATERN32"), (3, 3, "GAUSSIAN"),
                                         (2, 5, "EXPONENTIAL"), (3, 6, "MATERN52"),
                                         (2, 10, "EXPONENTIAL"), (2, 14, "MATERN32"),
                                         (1, 15, "GAUSSIAN")])
def test_gpu_matvec_against_oracle(cuda_device, precision, dim, p, kname):
    n = 20000
    P = uniform_cloud(n, dim, seed=p)
    x = np.random.default_rng(p).standard_normal((n, 32))
    ktype = {"EXPONENTIAL": 0, "MATERN32": 1, "MATERN52": 2, "GAUSSIAN": 3}[kname]
    O = oracle.OraclePlan(P, p=p, eta=0.8, min_leaf=64, interpolator="total_degree")
    assert O.n_far > 0
    y_ref, _ = O.action(ktype, 0.5, x)
    H = H2Matrix(CovarianceKernel(kname, 0.5), P, P, p, 0.8, min_leaf=64,
                 precision=precision, interpolator="total_degree")
    y = H.action(x)
    H.check_device_error()
    assert rel_err(y, y_ref) < TOL[precision]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_unsymmetric_total_degree(cuda_device, precision):
    Pr = sphere_cloud(6000, seed=11)
    Pc = sphere_cloud(9000, seed=12)
    x = np.random.default_rng(3).standard_normal((9000, 32))
    O = oracle.OraclePlan(Pr, Pc, p=4, eta=0.8, min_leaf=64, interpolator="total_degree")
    y_ref, _ = O.action(2, 0.3, x)
    H = H2Matrix(CovarianceKernel("MATERN52", 0.3), Pr, Pc, 4, 0.8, min_leaf=64,
                 precision=precision, interpolator="total_degree")
    assert rel_err(H.action(x), y_ref) < TOL[precision]


@pytest.mark.gpu
def test_gpu_adjoint_refuses_total_degree(cuda_device):
    P = uniform_cloud(3000, 3, seed=2)
    H = H2Matrix(CovarianceKernel("MATERN52", 0.3), P, P, 4, 0.8,
                 precision="fp64", interpolator="total_degree")
    import torch
    x = torch.randn(3000, 1, dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.FmcaError) as e:
        H.adjoint(x, x)
    assert e.value.status == ERR["FMCA_ERR_UNSUPPORTED"]


def test_nodes_match_the_lapack_golden_fixture():
    """DeMarchi nodes and invV against tests/golden/total_degree.json (scipy's
    Halton points, LAPACK's column-pivoted QR; gen_total_degree.py): the same
    pivots, coordinates within an ulp."""
    import json
    import os
    G = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                    "total_degree.json")))
    assert len(G) == 6
    for g in G.values():
        P = uniform_cloud(300, g["dim"], seed=1)
        H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, g["degree"], 0.8,
                     interpolator="total_degree")
        assert H.info["q"] == g["q"]
        nodes, invV = H.interpolation_nodes()
        assert np.abs(nodes - np.array(g["nodes"]).T).max() <= 4.5e-16
        if "invV" in g:
            ref = np.array(g["invV"])
            assert np.abs(invV - ref).max() <= 1e-13 * np.abs(ref).max()
