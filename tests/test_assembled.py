"""Assembled H2 matrix: stored far-field and near-field blocks.

The reference's H2Matrix(CT, mat_eval, eta) constructor (H2Matrix.h:53-66)
runs computeH2Matrix (H2MatrixBase.h:222-255), which evaluates and stores the
coupling matrix S of every admissible block and every dense block; its
operator* (H2MatrixBase.h:107-109, matrix_vector_product_impl.h:17-98)
multiplies with the stored blocks and full() (H2MatrixBase.h:155-158) forms
H * I.  Here computeH2Matrix stores the blocks on the GPU
(fmca_plan_assemble) and H * x streams them (fmca_matvec_assembled).

CPU: the byte count of fmca_plan_assembled_size against the block lists.
GPU (through the C ABI): the assembled product against the FP64 oracle
(FP64 to 1e-12, FP32 to 1e-5) and against the matrix-free product of the
same precision; full() against the dense oracle kernel matrix (the H2
compression error) and against H * x; the plan's device memory grows by
exactly the reported bytes and shrinks back on release; misuse is refused."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err, sphere_cloud, uniform_cloud
from fmca_gb300 import CovarianceKernel, FmcaError, H2Matrix, _lib

TOL = {"fp64": 1e-12, "fp32": 1e-5, "mixed": 1e-5}
ERR = {v: k for k, v in _lib.STATUS_NAMES.items()}


def expected_bytes(H, precision):
    """Stored elements from the block lists: every group (the nodes of a row
    cluster, the points of a row leaf; chunks of at most 256 targets) keeps
    (its sources) x (its targets rounded up to 4) values, plus one 8-byte
    offset per group."""
    q = H.info["q"]
    meta_r, _ = H.clusters(0)
    meta_c, _ = H.clusters(1)
    r4 = lambda t: (t + 3) // 4 * 4  # noqa: E731

    def rows(tc):
        return sum(r4(min(256, tc - o)) for o in range(0, tc, 256)), (tc + 255) // 256

    elems = groups = 0
    far_r, _ = H.blocks(0)
    nfar = np.bincount(far_r, minlength=H.info["row_clusters"])
    qr, qg = rows(q)
    for c in range(H.info["row_clusters"]):
        elems += int(nfar[c]) * q * qr
        groups += qg
    # dense blocks belong to the row leaves inside their row cluster (a dense
    # block may pair a leaf with a larger cluster on either side)
    is_leaf = np.ones(len(meta_r), bool)
    is_leaf[meta_r[:, 3][meta_r[:, 3] >= 0]] = False
    leaves = np.nonzero(is_leaf)[0]
    near_r, near_c = H.blocks(1)
    srcs = {}
    for r, c in zip(near_r, near_c):
        b, e = meta_r[r, 0], meta_r[r, 0] + meta_r[r, 1]
        for lf in leaves[(meta_r[leaves, 0] >= b) & (meta_r[leaves, 0] < e)]:
            srcs[lf] = srcs.get(lf, 0) + int(meta_c[c, 1])
    for lf, ns in srcs.items():
        lr, lg = rows(int(meta_r[lf, 1]))
        elems += ns * lr
        groups += lg
    return elems * (8 if precision == "fp64" else 4) + groups * 8


@pytest.mark.parametrize("p,leaf,n", [(3, 64, 3000), (2, 0, 2500), (4, 300, 2000)])
def test_assembled_size_counts_the_blocks(p, leaf, n):
    P = uniform_cloud(n, 3, seed=p)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.4), P, P, p, 0.8, min_leaf=leaf)
    for prec in ("fp64", "fp32", "mixed"):
        assert H.assembled_bytes(prec) == expected_bytes(H, prec)


def test_assembled_size_of_a_batched_plan():
    # a forest of clouds: the groups of every cloud, in one store
    rng = np.random.default_rng(12)
    clouds = [uniform_cloud(int(n), 3, seed=i) for i, n in enumerate(rng.integers(300, 2500, 4))]
    B = H2Matrix.batched(CovarianceKernel("MATERN32", 0.3), clouds, 3, 0.8)
    singles = [H2Matrix(CovarianceKernel("MATERN32", 0.3), P, P, 3, 0.8) for P in clouds]
    for prec in ("fp64", "fp32"):
        assert B.assembled_bytes(prec) == sum(S.assembled_bytes(prec) for S in singles)


def test_assembled_size_of_two_clouds():
    Pr = sphere_cloud(1500, seed=1)
    Pc = sphere_cloud(2200, seed=2)
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 0.5), Pr, Pc, 3, 0.8)
    assert H.assembled_bytes("fp32") == expected_bytes(H, "fp32")


@pytest.fixture(scope="module")
def case():
    P = uniform_cloud(6000, 3, seed=21)
    X = np.random.default_rng(21).standard_normal((6000, 40))
    O = oracle.OraclePlan(P, None, 3, 0.8, 64)
    Y_ref, _ = O.action(1, 0.45, X)
    return P, X, Y_ref


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_assembled_product_against_oracle(cuda_device, case, prec):
    import torch
    P, X, Y_ref = case
    H = H2Matrix(CovarianceKernel("MATERN32", 0.45), P, P, 3, 0.8, min_leaf=64, precision=prec)
    H.computeH2Matrix()
    assert H.assembled == prec
    torch.cuda.synchronize()
    for R in (1, 5, 8, 32, 40):
        x = torch.tensor(X[:, :R], device=cuda_device)
        y = H.mul(x)
        torch.cuda.synchronize()
        H.check_device_error()
        assert rel_err(y.cpu().numpy(), Y_ref[:, :R]) < TOL[prec], R
        y_mf = H.matvec(x, precision="fp64" if prec == "fp64" else "fp32")
        tol = 1e-13 if prec == "fp64" else 2e-6
        assert rel_err(y.cpu().numpy(), y_mf.cpu().numpy()) < tol, R
    # FP32 inputs, cluster order
    x32 = torch.tensor(X[:, :8], device=cuda_device, dtype=torch.float32)
    y32 = H.mul(x32)
    assert rel_err(y32.cpu().numpy(), Y_ref[:, :8]) < 1e-5
    yc = H.mul(x, order="cluster")
    assert yc.shape == (6000, 40)


@pytest.mark.gpu
def test_operator_mul_and_memory(cuda_device, case):
    import torch
    P, X, Y_ref = case
    H = H2Matrix(CovarianceKernel("MATERN32", 0.45), P, P, 3, 0.8, min_leaf=64, precision="fp64")
    with pytest.raises(FmcaError):
        H * X[:, :2]
    H.matvec(torch.tensor(X[:, :2], device=cuda_device))  # resident
    torch.cuda.synchronize()
    held = H.device_bytes()
    H.computeH2Matrix()
    torch.cuda.synchronize()
    assert H.device_bytes() - held == H.assembled_bytes("fp64")
    Y = H * X  # numpy in, numpy out (natural order)
    assert isinstance(Y, np.ndarray) and Y.shape == X.shape
    assert rel_err(Y, Y_ref) < 1e-12
    assert rel_err(H * X[:, 0], Y_ref[:, 0]) < 1e-12
    # FP64 blocks serve FP64 products only
    with pytest.raises(FmcaError) as e:
        H.mul(torch.tensor(X[:, :2], device=cuda_device), precision="fp32")
    assert e.value.status == ERR["FMCA_ERR_INVALID_ARGUMENT"]
    # a second assembly replaces the first, with another kernel
    H.computeH2Matrix(cov=CovarianceKernel("GAUSSIAN", 0.3))
    O = oracle.OraclePlan(P, None, 3, 0.8, 64)
    Yg, _ = O.action(3, 0.3, X[:, :3])
    assert rel_err(H * X[:, :3], Yg) < 1e-12
    assert H.device_bytes() - held == H.assembled_bytes("fp64")
    H.release_assembled()
    assert H.device_bytes() == held
    with pytest.raises(FmcaError):
        H.mul(torch.tensor(X[:, :2], device=cuda_device))


@pytest.mark.gpu
def test_full_matrix(cuda_device):
    n = 1500
    P = uniform_cloud(n, 3, seed=7)
    cov = CovarianceKernel("EXPONENTIAL", 0.8)
    H = H2Matrix(cov, P, P, 2, 0.8, min_leaf=32, precision="fp64")
    assert H.info["far_blocks"] > 0
    F_mf = H.full()
    H.computeH2Matrix()
    F = H.full()
    assert F.shape == (n, n)
    assert rel_err(F, F_mf) < 1e-13
    K = oracle.dense_matvec(0, 0.8, P, P, np.eye(n))
    e = rel_err(F, K)
    F_ref, _ = oracle.OraclePlan(P, None, 2, 0.8, 32).action(0, 0.8, np.eye(n))
    assert rel_err(F, F_ref) < 1e-12
    assert 1e-6 < e < 1e-3  # the H2 compression error at p = 2 (2.0e-4)
    assert abs(e - rel_err(F_ref, K)) < 1e-10
    x = np.random.default_rng(8).standard_normal((n, 3))
    assert rel_err(H * x, F @ x) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_assembled_two_clouds_and_total_degree(cuda_device, prec):
    import torch
    # unsymmetric (H2kernelActor-like) clouds, leaves above 256 points
    Pr = sphere_cloud(5000, seed=3)
    Pc = sphere_cloud(4000, seed=4)
    X = np.random.default_rng(5).standard_normal((4000, 9))
    H = H2Matrix(CovarianceKernel("MATERN52", 0.6), Pr, Pc, 3, 0.8, min_leaf=300, precision=prec)
    H.computeH2Matrix()
    y = H.mul(torch.tensor(X, device=cuda_device)).cpu().numpy()
    Y_ref, _ = oracle.OraclePlan(Pr, Pc, 3, 0.8, 300).action(2, 0.6, X)
    assert rel_err(y, Y_ref) < TOL[prec]
    # total-degree interpolation (the far field between two basis changes)
    P = uniform_cloud(5000, 3, seed=6)
    X = np.random.default_rng(6).standard_normal((5000, 32))
    H = H2Matrix(CovarianceKernel("GAUSSIAN", 0.3), P, P, 4, 0.8, min_leaf=64, precision=prec,
                 interpolator="total_degree")
    H.computeH2Matrix()
    y = H.mul(torch.tensor(X, device=cuda_device)).cpu().numpy()
    O = oracle.OraclePlan(P, p=4, eta=0.8, min_leaf=64, interpolator="total_degree")
    Y_ref, _ = O.action(3, 0.3, X)
    assert rel_err(y, Y_ref) < TOL[prec]
    H.check_device_error()


@pytest.mark.gpu
def test_assembled_batched_clouds(cuda_device):
    import torch
    rng = np.random.default_rng(11)
    clouds = [uniform_cloud(int(n), 3, seed=i) for i, n in enumerate(rng.integers(800, 4000, 5))]
    cov = CovarianceKernel("MATERN32", 0.3)
    B = H2Matrix.batched(cov, clouds, 3, 0.8, precision="fp32")
    B.computeH2Matrix()
    X = rng.standard_normal((B.rows(), 16))
    Y = B.mul(torch.tensor(X, device=cuda_device)).cpu().numpy()
    for i, P in enumerate(clouds):
        o, e = B.offsets[i], B.offsets[i + 1]
        Yi, _ = oracle.OraclePlan(P, None, 3, 0.8, 0).action(1, 0.3, X[o:e])
        assert rel_err(Y[o:e], Yi) < 1e-5, i


@pytest.mark.gpu
def test_assembled_stream_wait_runs_out(cuda_device, case):
    # the stream kernel's bounded waits: the stalled-wait hook makes the first
    # wait of every CTA run out; the next products are right again
    import torch
    P, X, Y_ref = case
    H = H2Matrix(CovarianceKernel("MATERN32", 0.45), P, P, 3, 0.8, min_leaf=64, precision="fp32")
    H.computeH2Matrix()
    x = torch.tensor(X[:, :8], device=cuda_device)
    H.mul(x)
    H.check_device_error()
    H.set_wait_limit(1_000_000)
    H.set_stalled_wait(True)
    H.mul(x)
    with pytest.raises(FmcaError) as e:
        H.check_device_error()
    assert e.value.status == ERR["FMCA_ERR_TIMEOUT"]
    H.set_stalled_wait(False)
    H.set_wait_limit(0)
    y = H.mul(x)
    H.check_device_error()
    assert rel_err(y.cpu().numpy(), Y_ref[:, :8]) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("n,dim", [(1, 3), (2, 3), (17, 3), (500, 1), (3000, 2)])
def test_assembled_small_and_low_dimensional(cuda_device, n, dim):
    # single points, a leaf-only tree, one and two dimensions
    import torch
    P = uniform_cloud(n, dim, seed=n + dim)
    X = np.random.default_rng(n).standard_normal((n, 3))
    cov = CovarianceKernel("MATERN52", 0.5)
    H = H2Matrix(cov, P, P, 3, 0.8, precision="fp64")
    assert H.assembled_bytes("fp64") == expected_bytes(H, "fp64")
    H.computeH2Matrix()
    y = H.mul(torch.tensor(X, device=cuda_device)).cpu().numpy()
    Y_ref, _ = oracle.OraclePlan(P, None, 3, 0.8, 0).action(2, 0.5, X)
    assert rel_err(y, Y_ref) < 1e-12
    H.check_device_error()
