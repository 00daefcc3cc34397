"""PyTorch autograd for the H2 product, for GP hyperparameter gradients.

``h2_matvec(H, x, l, sigma2, X)`` returns y = sigma2 * H2[k_l](X) x for an
``H2Matrix`` H built on one point cloud, differentiable with respect to x,
the length scale l, the variance sigma2 and the point coordinates X (dim x n).
The cluster tree, its boxes and the interpolation nodes stay those of H; a
changed X moves the points inside that frozen structure
(``fmca_plan_update_points``).  The backward pass calls the adjoint kernels
(``fmca_matvec_adjoint``): with g = dL/dy,
    dL/dx = K^T g = K g,  dL/dl = g^T H2[dk/dl] x,
    dL/dsigma2 = g^T H2 x,  dL/dX = d(g^T K x)/dX.
"""
from __future__ import annotations

import numpy as np
import torch

from .h2 import H2Matrix


class _H2Matvec(torch.autograd.Function):
    # Every forward records the state it ran with (point coordinates, l and
    # sigma2), and its backward puts that state back on H before the adjoint:
    # several forwards on one H may run before their backwards (for instance
    # two losses at different X summed into one objective), and each backward
    # must differentiate at its own forward's points.
    @staticmethod
    def forward(ctx, H: H2Matrix, precision, x, l, sigma2, X):
        if X is not None:
            H.update_points(X.detach().to(torch.float64).cpu().numpy())
        ctx.H = H
        ctx.precision = precision
        ctx.l, ctx.sigma2 = float(l), float(sigma2)
        ctx.points = H.current_points()
        ctx.X_meta = None if X is None else (X.dtype, X.device)
        H.cov.l, H.cov.sigma2 = ctx.l, ctx.sigma2
        ctx.save_for_backward(x)
        return H.matvec(x, precision=precision)

    @staticmethod
    def backward(ctx, gy):
        (x,) = ctx.saved_tensors
        H = ctx.H
        H.cov.l, H.cov.sigma2 = ctx.l, ctx.sigma2
        if ctx.points is not None and H.current_points() is not ctx.points:
            H.update_points(ctx.points)
        need_x = ctx.needs_input_grad[2]
        need_X = ctx.X_meta is not None and ctx.needs_input_grad[5]
        out = H.adjoint(x, gy.contiguous(), precision=ctx.precision, want_dX=need_X,
                        want_Ky=need_x)
        vals = out["values"].cpu()
        gx = out["Ky"] if need_x else None
        gl = vals[1] if ctx.needs_input_grad[3] else None
        gs = vals[2] if ctx.needs_input_grad[4] else None
        gX = None
        if need_X:
            dtype, device = ctx.X_meta
            gX = out["dX"].t().to(device=device, dtype=dtype)
        return None, None, gx, gl, gs, gX


def h2_matvec(H: H2Matrix, x: torch.Tensor, l=None, sigma2=None, X=None,
              precision: str | None = None) -> torch.Tensor:
    """Differentiable y = sigma2 * H2[k_l](X) x (see the module docstring)."""
    l = torch.as_tensor(H.cov.l if l is None else l, dtype=torch.float64)
    sigma2 = torch.as_tensor(H.cov.sigma2 if sigma2 is None else sigma2, dtype=torch.float64)
    if X is not None and tuple(X.shape) != (H.dim, H.rows()):
        raise ValueError("X must be dim x n")
    return _H2Matvec.apply(H, precision or H.precision, x, l, sigma2, X)


def dense_reference(kname: str, l, sigma2, X, x):
    """sigma2 * K(X, X) x with torch (for checks): the radial kernels of
    FMCA's CovarianceKernel, differentiable in every argument."""
    D = torch.cdist(X.t(), X.t())
    t = D / l
    if kname == "EXPONENTIAL":
        K = torch.exp(-t)
    elif kname == "MATERN32":
        a = np.sqrt(3.0) * t
        K = (1 + a) * torch.exp(-a)
    elif kname == "MATERN52":
        a = np.sqrt(5.0) * t
        K = (1 + a + a * a / 3) * torch.exp(-a)
    elif kname == "GAUSSIAN":
        K = torch.exp(-0.5 * t * t)
    else:
        raise ValueError(kname)
    return sigma2 * (K @ x)
