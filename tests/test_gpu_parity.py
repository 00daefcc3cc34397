"""GPU matvec against the FP64 oracle (same seeded inputs), through the C ABI.

Tolerances (relative 2-norm over all right-hand sides): FMCA_PREC_FP64 must
match the oracle to 1e-12; FMCA_PREC_FP32 (FP32 CUDA cores, FP32
accumulation) and FMCA_PREC_MIXED (FP32 kernel values, tensor-core
contractions on FP16 hi/lo splits, FP32 accumulation) to 1e-5.  The mixed
mode runs on the tensor cores for the bounded kernels with more than 16
right-hand sides and falls back to FP32 otherwise."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err, sphere_cloud, uniform_cloud
from fmca_gb300 import CovarianceKernel, H2Matrix

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-5, "mixed": 1e-5}
PRECS = ["fp64", "fp32", "mixed"]
KNAMES = ["EXPONENTIAL", "MATERN32", "MATERN52", "GAUSSIAN", "MATERN72", "MATERN92",
          "INVMULTIQUADRIC", "MULTIQUADRIC", "BIHARMONIC3D", "TRIHARMONIC3D"]
# kernel codes of the C ABI (FMCA_KERNEL_*)
KCODE = {**{k: i for i, k in enumerate(KNAMES)}, "BIHARMONIC2D": 14, "TPS2D": 15}


@pytest.fixture(scope="module")
def c1():
    # n = 1e4 uniform [0,1]^3 (seed 0), EXPONENTIAL l=1, p=3, eta=0.8, leaf 64
    P = uniform_cloud(10000, 3, seed=0)
    x = np.random.default_rng(0).standard_normal(10000)
    O = oracle.OraclePlan(P, None, 3, 0.8, 64)
    y_ref, _ = O.action(0, 1.0, x)
    return P, x, y_ref


@pytest.mark.parametrize("precision", PRECS)
def test_c1_against_oracle(cuda_device, c1, precision):
    P, x, y_ref = c1
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, 3, 0.8, min_leaf=64,
                 precision=precision)
    y = H.action(x)
    assert rel_err(y, y_ref) < TOL[precision]
    H.check_device_error()


def test_c1_against_dense(cuda_device, c1):
    # the GPU product has the oracle's compression error w.r.t. dense K x
    P, x, y_ref = c1
    yd = oracle.dense_matvec(0, 1.0, P, P, x)
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, 3, 0.8, min_leaf=64,
                 precision="fp64")
    y = H.action(x)
    e_gpu, e_ref = rel_err(y, yd), rel_err(y_ref, yd)
    assert e_ref < 1e-4
    assert abs(e_gpu - e_ref) < 1e-10


@pytest.mark.parametrize("kname", KNAMES)
@pytest.mark.parametrize("precision", PRECS)
def test_all_kernels(cuda_device, kname, precision):
    # 20 right-hand sides: the mixed mode takes the tensor-core path
    P = uniform_cloud(6000, 3, seed=11)
    X = np.random.default_rng(11).standard_normal((6000, 20))
    kt = KNAMES.index(kname)
    O = oracle.OraclePlan(P, None, 3, 0.8, 32)
    Y_ref, _ = O.action(kt, 0.7, X, c=0.9)
    H = H2Matrix(CovarianceKernel(kname, 0.7, 0.9), P, P, 3, 0.8, min_leaf=32,
                 precision=precision)
    assert rel_err(H.action(X), Y_ref) < TOL[precision]


@pytest.mark.parametrize("kname", ["BIHARMONIC2D", "TPS2D"])
@pytest.mark.parametrize("precision", PRECS)
def test_thin_plate_kernels_in_2d(cuda_device, kname, precision):
    # the thin-plate kernels of CovarianceKernel.h:56-59 and 117-118 (unbounded:
    # the mixed precision takes the FP32 CUDA-core path), 2-D, 24 right-hand
    # sides; tps: r^2 log r changes sign at r = 1, so the cloud spans [0, 3]^2
    P = uniform_cloud(8000, 2, seed=13) * 3.0
    X = np.random.default_rng(13).standard_normal((8000, 24))
    Y_ref, _ = oracle.OraclePlan(P, None, 5, 0.8, 32).action(KCODE[kname], 0.7, X)
    H = H2Matrix(CovarianceKernel(kname, 0.7), P, P, 5, 0.8, min_leaf=32, precision=precision)
    assert rel_err(H.action(X), Y_ref) < TOL[precision]
    H.check_device_error()


@pytest.mark.parametrize("kname", ["EXPONENTIAL", "MATERN52", "MATERN72", "MATERN92", "GAUSSIAN"])
def test_kernels_on_tensor_grids(cuda_device, kname):
    # 3-D, degree 4, 32 right-hand sides: the compile-time kernel values of
    # the tensor-core kernel sums, near field and sibling-paired grid far
    # field
    P = uniform_cloud(20000, 3, seed=12)
    X = np.random.default_rng(12).standard_normal((20000, 32))
    kt = KNAMES.index(kname)
    Y_ref, _ = oracle.OraclePlan(P, None, 4, 0.8, 128).action(kt, 0.4, X)
    H = H2Matrix(CovarianceKernel(kname, 0.4), P, P, 4, 0.8, min_leaf=128, precision="mixed")
    assert rel_err(H.action(X), Y_ref) < TOL["mixed"]


@pytest.mark.parametrize("R", [1, 2, 7, 8, 9, 16, 17, 32, 33, 64, 70])
@pytest.mark.parametrize("precision", PRECS)
def test_rhs_counts(cuda_device, R, precision):
    P = uniform_cloud(5000, 3, seed=R)
    X = np.random.default_rng(R).standard_normal((5000, R))
    O = oracle.OraclePlan(P, None, 4, 0.8, 0)
    Y_ref, _ = O.action(1, 0.5, X)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 4, 0.8, precision=precision)
    assert rel_err(H.action(X), Y_ref) < TOL[precision]


@pytest.mark.parametrize("precision", PRECS)
def test_unsymmetric_sphere(cuda_device, precision):
    Pr = sphere_cloud(7000, seed=1)
    Pc = sphere_cloud(4000, seed=2)
    X = np.random.default_rng(2).standard_normal((4000, 24))
    O = oracle.OraclePlan(Pr, Pc, 4, 0.8, 96)
    Y_ref, _ = O.action(2, 0.3, X, sigma2=1.7)
    H = H2Matrix(CovarianceKernel("MATERN52", 0.3, sigma2=1.7), Pr, Pc, 4, 0.8, min_leaf=96,
                 precision=precision)
    assert rel_err(H.action(X), Y_ref) < TOL[precision]


@pytest.mark.parametrize("precision", PRECS)
def test_two_dimensional_aniso(cuda_device, precision):
    P = uniform_cloud(20000, 2, seed=4)
    P[0] *= 4
    x = np.random.default_rng(4).choice([-1.0, 1.0], size=(20000, 64))
    O = oracle.OraclePlan(P, None, 5, 0.6, 128)
    Y_ref, _ = O.action(0, 0.1, x)
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 0.1), P, P, 5, 0.6, min_leaf=128,
                 precision=precision)
    assert rel_err(H.action(x), Y_ref) < TOL[precision]


@pytest.mark.parametrize("precision", PRECS)
def test_large_leaves_and_one_dim(cuda_device, precision):
    # leaves above the 256-target group size, and d = 1
    P = uniform_cloud(6000, 3, seed=8)
    x = np.random.default_rng(8).standard_normal((6000, 20))
    O = oracle.OraclePlan(P, None, 2, 0.8, 400)
    y_ref, _ = O.action(3, 0.2, x)
    H = H2Matrix(CovarianceKernel("GAUSSIAN", 0.2), P, P, 2, 0.8, min_leaf=400,
                 precision=precision)
    assert rel_err(H.action(x), y_ref) < TOL[precision]
    P1 = uniform_cloud(3000, 1, seed=8)
    x1 = np.random.default_rng(9).standard_normal((3000, 18))
    O1 = oracle.OraclePlan(P1, None, 6, 0.8, 0)
    y1_ref, _ = O1.action(1, 0.05, x1)
    H1 = H2Matrix(CovarianceKernel("MATERN32", 0.05), P1, P1, 6, 0.8, precision=precision)
    assert rel_err(H1.action(x1), y1_ref) < TOL[precision]


def test_tiny_clouds(cuda_device):
    for n in (1, 2, 17):
        P = uniform_cloud(n, 3, seed=n)
        x = np.random.default_rng(n).standard_normal(n)
        O = oracle.OraclePlan(P, None, 2, 0.8, 0)
        y_ref, _ = O.action(0, 1.0, x)
        for prec in PRECS:
            H = H2Matrix(CovarianceKernel("EXPONENTIAL"), P, P, 2, 0.8, precision=prec)
            assert rel_err(H.action(x), y_ref) < TOL[prec]
            X = np.tile(x[:, None], (1, 20)) * np.arange(1, 21)
            Y_ref = y_ref[:, None] * np.arange(1, 21)
            assert rel_err(H.action(X), Y_ref) < TOL[prec]


def test_torch_device_api(cuda_device):
    import torch
    P = uniform_cloud(8000, 3, seed=21)
    X = np.random.default_rng(21).standard_normal((8000, 16))
    O = oracle.OraclePlan(P, None, 3, 0.8, 0)
    Y_ref, _ = O.action(1, 0.4, X)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.4), P, P, 3, 0.8)
    Xt = torch.tensor(X, device=cuda_device)
    for prec in PRECS:
        y64 = H.matvec(Xt, precision=prec)                       # row-major (n, R)
        assert rel_err(y64.cpu().numpy(), Y_ref) < TOL[prec]
        Xf = Xt.t().contiguous().t()                              # column-major strides
        y_cm = H.matvec(Xf, precision=prec)
        assert rel_err(y_cm.cpu().numpy(), Y_ref) < TOL[prec]
    y32 = H.matvec(Xt.float(), precision="mixed")
    assert y32.dtype == torch.float32
    assert rel_err(y32.double().cpu().numpy(), Y_ref) < 2e-5
    # cluster order in and out: y_c = K_c x_c
    pr, pc = H.rindices(), H.cindices()
    Xc = Xt[torch.as_tensor(pc.astype(np.int64), device=cuda_device)]
    yc = H.matvec(Xc, precision="fp64", order="cluster")
    assert rel_err(yc.cpu().numpy(), Y_ref[pr.astype(np.int64)]) < 1e-12
    # CPU tensors go through the device and come back
    yt = H.action(torch.tensor(X))
    assert yt.device.type == "cpu" and rel_err(yt.numpy(), Y_ref) < TOL["mixed"]
    torch.cuda.synchronize()
    H.check_device_error()


def test_dense_kernel_eval(cuda_device):
    rng = np.random.default_rng(0)
    PR, PC = rng.random((3, 50)), rng.random((3, 40))
    for kname, kt in KCODE.items():
        K = CovarianceKernel(kname, 0.6, 0.8).eval(PR, PC)
        r = np.linalg.norm(PR[:, :, None] - PC[:, None, :], axis=0)
        ref = np.vectorize(lambda t: oracle.kernel(kt, 0.6, t, c=0.8))(r)
        # the thin-plate kernels cross zero at r = l (r = 1 for TPS2D), where a
        # relative tolerance would compare the rounding of two distances
        assert np.allclose(K, ref, rtol=1e-13, atol=1e-14 * np.abs(ref).max()), kname


@pytest.mark.parametrize("scale", [1e-30, 1e-6, 1.0, 1e8, 1e30])
def test_mixed_scaling_of_magnitudes(cuda_device, scale):
    # the tensor-core path scales right-hand sides and moments by powers of
    # two; results must not depend on the magnitude of x
    P = uniform_cloud(8000, 3, seed=31)
    rng = np.random.default_rng(31)
    X = rng.standard_normal((8000, 32))
    X[:, 3] = 1.0                 # constant column: large moments
    X[:, 5] = 0.0                 # zero column
    X[:100, 7] *= 1e6             # a few dominant entries
    O = oracle.OraclePlan(P, None, 4, 0.8, 0)
    Y_ref, _ = O.action(1, 0.3, X * scale)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.3), P, P, 4, 0.8, precision="mixed")
    Y = H.action(X * scale)
    assert np.all(Y[:, 5] == 0.0)
    for r in range(32):
        if r == 5:
            continue
        assert rel_err(Y[:, r], Y_ref[:, r]) < 1e-5, r


@pytest.mark.parametrize("kname", ["EXPONENTIAL", "MATERN32", "MATERN52", "GAUSSIAN",
                                   "MATERN72"])
def test_mixed_zero_and_positive_moment_regions(cuda_device, kname):
    # x vanishes on half of the cube (clusters without moments) and is
    # positive on the other half (large moments): each far group scales its
    # sources by its own largest moment exponent
    n = 20000
    P = uniform_cloud(n, 3, seed=41)
    rng = np.random.default_rng(41)
    X = 1.0 + 0.1 * rng.standard_normal((n, 32))
    X[P[0] < 0.5, :] = 0.0
    X[:, 1] = np.where(P[0] < 0.5, 0.0, 1e-3)
    X[:, 2] = np.where(P[1] < 0.25, 1e4, 1.0)
    kt = KNAMES.index(kname)
    O = oracle.OraclePlan(P, None, 4, 0.8, 0)
    Y_ref, _ = O.action(kt, 0.2, X)
    H = H2Matrix(CovarianceKernel(kname, 0.2), P, P, 4, 0.8, precision="mixed")
    Y = H.action(X)
    for r in range(32):
        assert rel_err(Y[:, r], Y_ref[:, r]) < 1e-5, r
    H.check_device_error()


def test_mixed_uses_tensor_core_kernel_count(cuda_device):
    # the mixed path launches the column-maximum, point-pair and moment-scale
    # kernels (three more launches than the FP32 path for one chunk)
    P = uniform_cloud(5000, 3, seed=2)
    X = np.random.default_rng(2).standard_normal((5000, 32))
    H = H2Matrix(CovarianceKernel("MATERN32", 0.3), P, P, 3, 0.8)
    import torch
    H.set_profiling(True)
    H.matvec(torch.tensor(X, device=cuda_device), precision="fp32")
    _, n32 = H.profile()
    H.matvec(torch.tensor(X, device=cuda_device), precision="mixed")
    stages, nmx = H.profile()
    assert nmx == n32 + 3
    assert stages["near"] > 0 and stages["far"] > 0


@pytest.mark.parametrize("dim,p", [(1, 4), (2, 3), (2, 4), (2, 6), (2, 7), (3, 3), (3, 5)])
def test_mixed_interpolation_orders(cuda_device, dim, p):
    # the sum-factorised transfers are compiled per (dimension, p + 1):
    # 2-D with 4..8 and 3-D with 4..6 nodes per dimension; 1-D takes the
    # dense transfer kernel
    n = 4000
    P = uniform_cloud(n, dim, seed=50 + 10 * dim + p)
    X = np.random.default_rng(p).standard_normal((n, 32))
    O = oracle.OraclePlan(P, None, p, 0.8, 0)
    Y_ref, _ = O.action(1, 0.5, X)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, p, 0.8, precision="mixed")
    assert rel_err(H.action(X), Y_ref) < 1e-5
    H.check_device_error()


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("dim,p", [(2, 7), (3, 5), (2, 2), (3, 2), (3, 6)])
def test_gaussian_far_field_as_kronecker_products(cuda_device, prec, dim, p):
    # GAUSSIAN far fields on tensor-product nodes are Kronecker products of
    # 1-D factors (grids of 3..8 nodes per dimension in 2-D, 3..6 in 3-D;
    # p = 6 in 3-D, 7 nodes, takes the kernel sum); in mixed precision the
    # tensor-core kernel sum stays a choice of the tuned configuration
    import torch
    n, R = 12000, 32
    P = uniform_cloud(n, dim, seed=10 * dim + p)
    X = np.random.default_rng(p).standard_normal((n, R))
    O = oracle.OraclePlan(P, None, p, 0.8, 0)
    assert O.n_far > 0
    Y_ref, _ = O.action(3, 0.3, X)
    H = H2Matrix(CovarianceKernel("GAUSSIAN", 0.3), P, P, p, 0.8, precision=prec)
    x = torch.tensor(X, device=cuda_device)
    y = H.matvec(x).cpu().numpy()
    H.check_device_error()
    assert rel_err(y, Y_ref) < TOL[prec]
    if prec == "mixed":
        cfg = H.tuned_config(R)
        assert cfg["far_kron"] == 1
        cfg["far_kron"] = 0
        H.set_tuned_config(R, cfg)
        y2 = H.matvec(x).cpu().numpy()
        H.check_device_error()
        assert rel_err(y2, Y_ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
@pytest.mark.parametrize("R", [1, 5, 20, 40])
@pytest.mark.parametrize("dim,p", [(3, 3), (2, 4)])
def test_gaussian_kronecker_column_counts(cuda_device, prec, R, dim, p):
    # the Kronecker far field holds 1, 8 or 32 right-hand sides per source
    # cluster (32, 4 or 1 clusters per warp step), some of them unused; 40
    # takes two launches, the second from column 32
    import torch
    n = 9000
    P = uniform_cloud(n, dim, seed=70 + 10 * dim + R)
    X = np.random.default_rng(R).standard_normal((n, R))
    O = oracle.OraclePlan(P, None, p, 0.8, 0)
    assert O.n_far > 0
    Y_ref, _ = O.action(3, 0.3, X)
    H = H2Matrix(CovarianceKernel("GAUSSIAN", 0.3), P, P, p, 0.8, precision=prec)
    y = H.matvec(torch.tensor(X, device=cuda_device)).cpu().numpy()
    H.check_device_error()
    assert rel_err(y, Y_ref) < TOL[prec]
