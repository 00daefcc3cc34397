"""Adjoint of the H2 product: gradients of f = sum_r y_r^T K x_r with respect
to the length scale, the variance and the point coordinates (tree, boxes and
interpolation nodes fixed).

CPU: the oracle's adjoint against central finite differences of the
oracle's own FP64 product with the points moved inside the frozen structure
(1e-6), against finite differences in l, and against dense FP64 torch
autograd up to the compression error.
GPU: the CUDA adjoint against the oracle (FP64: 1e-10), against central
finite differences (h = 1e-4) of the GPU FP64 product with frozen structure
(1e-6), and in FP32 / mixed precision against the FP64 oracle (1e-5 for the
values, 1e-4 for the point gradient)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err, sphere_cloud, uniform_cloud

KNAMES = ["EXPONENTIAL", "MATERN32", "MATERN52", "GAUSSIAN"]


def _problem(n=1500, R=3, seed=0, sphere=False):
    P = sphere_cloud(n, seed) if sphere else uniform_cloud(n, 3, seed)
    rng = np.random.default_rng(seed + 100)
    return P, rng.standard_normal((n, R)), rng.standard_normal((n, R))


@pytest.mark.parametrize("kt", range(4))
def test_oracle_adjoint_against_dense_autograd(kt):
    # dense FP64 torch autograd of y^T K(l, sigma2, X) x; the H2 gradient
    # differs by the compression error (p = 3, with far blocks present)
    torch = pytest.importorskip("torch")
    from fmca_gb300.autograd import dense_reference
    P, x, y = _problem(3000, 2, seed=kt)
    l, s2 = 0.4, 1.3
    O = oracle.OraclePlan(P, None, 3, 0.8, 16)
    assert O.n_far > 0
    vals, dX = oracle.adjoint(O, kt, l, x, y, sigma2=s2)
    Xt = torch.tensor(P, requires_grad=True)
    lt = torch.tensor(l, requires_grad=True, dtype=torch.float64)
    st = torch.tensor(s2, requires_grad=True, dtype=torch.float64)
    f = (torch.tensor(y) * dense_reference(KNAMES[kt], lt, st, Xt, torch.tensor(x))).sum()
    f.backward()
    assert abs(vals[0] - f.item()) / abs(f.item()) < 1e-3
    assert abs(vals[1] - lt.grad.item()) / abs(lt.grad.item()) < 2e-3
    assert abs(vals[2] - st.grad.item()) / abs(st.grad.item()) < 1e-3
    assert rel_err(dX, Xt.grad.numpy().T) < 5e-3


@pytest.mark.parametrize("kt", range(4))
def test_oracle_adjoint_against_finite_differences(kt):
    # central differences of the oracle's own H2 product with the points
    # moved inside the frozen structure (about 4000 far blocks)
    P, x, y = _problem(6000, 2, seed=kt + 20)
    O = oracle.OraclePlan(P, None, 2, 0.8, 0)
    assert O.n_far > 1000
    vals, dX = oracle.adjoint(O, kt, 0.3, x, y, sigma2=1.2)
    rng = np.random.default_rng(kt)
    h = 1e-5
    for _ in range(4):
        i, d = int(rng.integers(0, 6000)), int(rng.integers(0, 3))
        Pp, Pm = P.copy(), P.copy()
        Pp[d, i] += h
        Pm[d, i] -= h
        O.update_points(Pp)
        fp = np.sum(y * O.action(kt, 0.3, x, sigma2=1.2)[0])
        O.update_points(Pm)
        fm = np.sum(y * O.action(kt, 0.3, x, sigma2=1.2)[0])
        O.update_points(P)
        fd = (fp - fm) / (2 * h)
        assert abs(dX[i, d] - fd) <= 1e-6 * max(1.0, abs(fd)), (i, d)


def test_oracle_dl_against_finite_differences():
    P, x, y = _problem(1500, 2, seed=7)
    O = oracle.OraclePlan(P, None, 3, 0.8, 0)
    vals, _ = oracle.adjoint(O, 1, 0.3, x, y, sigma2=1.0)
    h = 1e-4 * 0.3
    fp, _ = O.action(1, 0.3 + h, x)
    fm, _ = O.action(1, 0.3 - h, x)
    fd = (np.sum(y * fp) - np.sum(y * fm)) / (2 * h)
    assert abs(vals[1] - fd) / abs(fd) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("kname", KNAMES)
def test_gpu_adjoint_against_oracle(cuda_device, kname):
    import torch
    from fmca_gb300 import CovarianceKernel, H2Matrix
    kt = KNAMES.index(kname)
    P, x, y = _problem(6000, 4, seed=kt + 3)
    l, s2 = 0.35, 0.8
    O = oracle.OraclePlan(P, None, 3, 0.8, 0)
    assert O.n_far > 1000
    vals_ref, dX_ref = oracle.adjoint(O, kt, l, x, y, sigma2=s2)
    H = H2Matrix(CovarianceKernel(kname, l, sigma2=s2), P, P, 3, 0.8)
    xt = torch.tensor(x, device=cuda_device)
    yt = torch.tensor(y, device=cuda_device)
    out = H.adjoint(xt, yt, precision="fp64", want_Kx=True, want_Ky=True)
    vals = out["values"].cpu().numpy()
    assert np.allclose(vals, vals_ref, rtol=1e-10, atol=0)
    assert rel_err(out["dX"].cpu().numpy(), dX_ref) < 1e-10
    Kx_ref, _ = O.action(kt, l, x, sigma2=s2)
    Ky_ref, _ = O.action(kt, l, y, sigma2=s2)
    assert rel_err(out["Kx"].cpu().numpy(), Kx_ref) < 1e-12
    assert rel_err(out["Ky"].cpu().numpy(), Ky_ref) < 1e-12
    # the lower precisions against the FP64 adjoint
    for prec in ("fp32", "mixed"):
        o = H.adjoint(xt, yt, precision=prec)
        v = o["values"].cpu().numpy()
        assert np.allclose(v, vals_ref, rtol=1e-5, atol=0), prec
        assert rel_err(o["dX"].cpu().numpy(), dX_ref) < 1e-4, prec
    H.check_device_error()


@pytest.mark.gpu
def test_gpu_adjoint_mixed_tensor_core_path(cuda_device):
    # 24 right-hand sides: the mixed products run on the tensor cores
    import torch
    from fmca_gb300 import CovarianceKernel, H2Matrix
    P, x, y = _problem(8000, 24, seed=11, sphere=True)
    O = oracle.OraclePlan(P, None, 3, 0.8, 0)
    assert O.n_far > 1000
    vals_ref, dX_ref = oracle.adjoint(O, 2, 0.3, x, y, sigma2=1.0)
    H = H2Matrix(CovarianceKernel("MATERN52", 0.3), P, P, 3, 0.8)
    out = H.adjoint(torch.tensor(x, device=cuda_device), torch.tensor(y, device=cuda_device),
                    precision="mixed")
    assert np.allclose(out["values"].cpu().numpy(), vals_ref, rtol=1e-5, atol=0)
    assert rel_err(out["dX"].cpu().numpy(), dX_ref) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("R", [1, 5])
def test_gpu_adjoint_few_rhs_on_padded_tensor_cores(cuda_device, R):
    # fewer than 17 right-hand sides with the tensor-core path set for the
    # key (as the autotuner may choose it): the products run on 32 padded
    # columns and the gradient terms read only the R occupied ones
    import torch
    from fmca_gb300 import CovarianceKernel, H2Matrix
    P, x, y = _problem(8000, R, seed=13, sphere=True)
    O = oracle.OraclePlan(P, None, 4, 0.8, 0)
    vals_ref, dX_ref = oracle.adjoint(O, 2, 0.3, x, y, sigma2=1.0)
    H = H2Matrix(CovarianceKernel("MATERN52", 0.3), P, P, 4, 0.8)
    xt, yt = torch.tensor(x, device=cuda_device), torch.tensor(y, device=cuda_device)
    H.matvec(xt)  # resident
    H.set_tuned_config(R, {**H.tuned_config(R), "small_r_tensor": 1})
    out = H.adjoint(xt, yt, precision="mixed")
    H.check_device_error()
    # f and its derivatives are single scalars summed over few columns: the
    # mixed path's ~1e-6 relative error of the products grows by their
    # cancellation (df/dl 3e-5 here at R = 1, the CUDA-core path alike)
    assert np.allclose(out["values"].cpu().numpy(), vals_ref, rtol=1e-4, atol=0)
    assert rel_err(out["dX"].cpu().numpy(), dX_ref) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("kname", ["MATERN32", "MATERN52", "GAUSSIAN"])
def test_gpu_adjoint_against_finite_differences(cuda_device, kname):
    # central differences (h = 1e-4) of the GPU FP64 product with the tree,
    # boxes and nodes frozen
    import torch
    from fmca_gb300 import CovarianceKernel, H2Matrix
    P, x, y = _problem(6000, 2, seed=5)
    l = 0.3
    H = H2Matrix(CovarianceKernel(kname, l), P, P, 2, 0.8, precision="fp64")
    assert H.info["far_blocks"] > 1000
    xt = torch.tensor(x, device=cuda_device)
    yt = torch.tensor(y, device=cuda_device)
    out = H.adjoint(xt, yt)
    vals = out["values"].cpu().numpy()
    dX = out["dX"].cpu().numpy()

    def f(cov_l=l, P_=None):
        if P_ is not None:
            H.update_points(P_)
        H.cov.l = cov_l
        v = float((yt * H.matvec(xt)).sum())
        H.cov.l = l
        return v

    h = 1e-4
    fd_l = (f(l * (1 + h)) - f(l * (1 - h))) / (2 * l * h)
    assert abs(vals[1] - fd_l) / abs(fd_l) < 1e-6
    rng = np.random.default_rng(1)
    for _ in range(4):
        i, d = int(rng.integers(0, 6000)), int(rng.integers(0, 3))
        Pp, Pm = P.copy(), P.copy()
        Pp[d, i] += h
        Pm[d, i] -= h
        fd = (f(P_=Pp) - f(P_=Pm)) / (2 * h)
        H.update_points(P)
        assert abs(dX[i, d] - fd) <= 1e-6 * max(1.0, abs(fd)), (i, d, dX[i, d], fd)


@pytest.mark.gpu
def test_autograd_function(cuda_device):
    import torch
    from fmca_gb300 import CovarianceKernel, H2Matrix
    from fmca_gb300.autograd import h2_matvec
    P, x, y = _problem(5000, 3, seed=9)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.4), P, P, 3, 0.8, precision="fp64")
    xt = torch.tensor(x, device=cuda_device, requires_grad=True)
    lt = torch.tensor(0.4, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(1.5, dtype=torch.float64, requires_grad=True)
    Xt = torch.tensor(P, requires_grad=True)
    yt = torch.tensor(y, device=cuda_device)
    f = (yt * h2_matvec(H, xt, lt, st, Xt)).sum()
    f.backward()
    O = oracle.OraclePlan(P, None, 3, 0.8, 0)
    vals_ref, dX_ref = oracle.adjoint(O, 1, 0.4, x, y, sigma2=1.5)
    assert abs(f.item() - vals_ref[0]) / abs(vals_ref[0]) < 1e-12
    assert abs(lt.grad.item() - vals_ref[1]) / abs(vals_ref[1]) < 1e-10
    assert abs(st.grad.item() - vals_ref[2]) / abs(vals_ref[2]) < 1e-10
    assert rel_err(Xt.grad.numpy(), dX_ref.T) < 1e-10
    Ky_ref, _ = O.action(1, 0.4, y, sigma2=1.5)
    assert rel_err(xt.grad.cpu().numpy(), Ky_ref) < 1e-12


@pytest.mark.gpu
def test_autograd_two_forwards_before_their_backwards(cuda_device):
    # two forwards on one H at different points and length scales, then both
    # backwards: each backward must differentiate at its own forward's state
    import torch
    from fmca_gb300 import CovarianceKernel, H2Matrix
    from fmca_gb300.autograd import dense_reference, h2_matvec
    P, x, y = _problem(4000, 2, seed=11)
    P2 = P + 1e-3 * np.random.default_rng(12).standard_normal(P.shape)
    H = H2Matrix(CovarianceKernel("MATERN52", 0.4), P, P, 4, 0.8, precision="fp64")

    def leaf(v, dev=None):
        return torch.tensor(v, dtype=torch.float64, device=dev, requires_grad=True)

    def grads(X, l, s2):
        xt, lt, st, Xt = leaf(x, cuda_device), leaf(l), leaf(s2), leaf(X)
        f = (torch.tensor(y, device=cuda_device) * h2_matvec(H, xt, lt, st, Xt)).sum()
        return f, (xt, lt, st, Xt)

    # one at a time
    ref = []
    for X, l, s2 in ((P, 0.4, 1.5), (P2, 0.3, 0.7)):
        f, leaves = grads(X, l, s2)
        f.backward()
        ref.append((f.item(), [t.grad.cpu().numpy().copy() for t in leaves]))
    # both forwards first, then the backwards in reverse order
    f1, a = grads(P, 0.4, 1.5)
    f2, b = grads(P2, 0.3, 0.7)
    f2.backward()
    f1.backward()
    for (fr, gr), f, leaves in zip(ref, (f1, f2), (a, b)):
        assert abs(f.item() - fr) <= 1e-13 * abs(fr)
        for t, g in zip(leaves, gr):
            assert rel_err(t.grad.cpu().numpy(), g) <= 1e-12
    # and the second state against dense FP64 autograd (compression error)
    Xt, lt, st = leaf(P2), leaf(0.3), leaf(0.7)
    fd = (torch.tensor(y) * dense_reference("MATERN52", lt, st, Xt, torch.tensor(x))).sum()
    fd.backward()
    assert abs(f2.item() - fd.item()) / abs(fd.item()) < 1e-4
    assert abs(b[1].grad.item() - lt.grad.item()) / abs(lt.grad.item()) < 1e-3
    assert rel_err(b[3].grad.cpu().numpy(), Xt.grad.numpy()) < 1e-3


@pytest.mark.gpu
def test_c4_small_case_against_dense_autograd_and_differences(cuda_device):
    # the gradient workload's own checks at its reduced size: n = 5000 points
    # on S^2, MATERN52 l = 0.3, sigma2 = 1, p = 4, eta = 0.8, leaf 96
    # (effective 125), x, y ~ N(0, 1) drawn in float32.  The GPU gradients
    # (FP64 and mixed) against dense FP64 torch autograd of y^T K x (up to
    # the H2 compression error, 7e-6 in f and 2e-5 in dX here) and the FP64
    # ones against central differences with h = 1e-4 (1e-6)
    import torch
    from fmca_gb300 import CovarianceKernel, H2Matrix
    from fmca_gb300.autograd import dense_reference
    n, l = 5000, 0.3
    P = sphere_cloud(n, seed=0)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((n, 1)).astype(np.float32)
    y = rng.standard_normal((n, 1)).astype(np.float32)
    Xt = torch.tensor(P, device=cuda_device, requires_grad=True)
    lt = torch.tensor(l, dtype=torch.float64, device=cuda_device, requires_grad=True)
    st = torch.tensor(1.0, dtype=torch.float64, device=cuda_device, requires_grad=True)
    fd_ = (torch.tensor(y, dtype=torch.float64, device=cuda_device) *
           dense_reference("MATERN52", lt, st, Xt,
                           torch.tensor(x, dtype=torch.float64, device=cuda_device))).sum()
    fd_.backward()
    dense = {"f": fd_.item(), "dl": lt.grad.item(), "ds": st.grad.item(),
             "dX": Xt.grad.cpu().numpy().T}
    H = H2Matrix(CovarianceKernel("MATERN52", l), P, P, 4, 0.8, min_leaf=96, precision="fp64")
    assert H.info["far_blocks"] > 0
    got = {}
    for prec, dt in (("fp64", torch.float64), ("mixed", torch.float32)):
        out = H.adjoint(torch.tensor(x, dtype=dt, device=cuda_device),
                        torch.tensor(y, dtype=dt, device=cuda_device), precision=prec)
        v = out["values"].cpu().numpy()
        got[prec] = {"f": v[0], "dl": v[1], "ds": v[2],
                     "dX": out["dX"].double().cpu().numpy()}
        H.check_device_error()
    bound = {"fp64": {"f": 2e-5, "dl": 4e-5, "ds": 2e-5, "dX": 6e-5},
             "mixed": {"f": 1e-4, "dl": 1e-4, "ds": 1e-4, "dX": 1e-4}}
    for prec in ("fp64", "mixed"):
        for k in ("f", "dl", "ds"):
            assert abs(got[prec][k] - dense[k]) / abs(dense[k]) < bound[prec][k], (prec, k)
        assert rel_err(got[prec]["dX"], dense["dX"]) < bound[prec]["dX"], prec
    # central differences of the GPU FP64 product (tree, boxes, nodes frozen)
    xt = torch.tensor(x, dtype=torch.float64, device=cuda_device)
    yt = torch.tensor(y, dtype=torch.float64, device=cuda_device)

    def f(cov_l=l, P_=None):
        if P_ is not None:
            H.update_points(P_)
        H.cov.l = cov_l
        v = float((yt * H.matvec(xt)).sum())
        H.cov.l = l
        return v

    h = 1e-4
    fd_l = (f(l * (1 + h)) - f(l * (1 - h))) / (2 * l * h)
    assert abs(got["fp64"]["dl"] - fd_l) / abs(fd_l) < 1e-6
    for _ in range(4):
        i, d = int(rng.integers(0, n)), int(rng.integers(0, 3))
        Pp, Pm = P.copy(), P.copy()
        Pp[d, i] += h
        Pm[d, i] -= h
        fd = (f(P_=Pp) - f(P_=Pm)) / (2 * h)
        H.update_points(P)
        assert abs(got["fp64"]["dX"][i, d] - fd) <= 1e-6 * max(1.0, abs(fd)), (i, d)
