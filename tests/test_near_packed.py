"""Near field of the tensor-core kernel sum on packed groups: the rows of up
to two consecutive row leaves per CTA (128 targets, one half) over the union
of the leaves' source intervals, every target masked to its own leaf's
sources (H2MatrixBase.h:143-146: the dense blocks of one row leaf).

GPU: the packed launch, forced through the tuned configuration, against the
FP64 oracle and against the launch of one leaf per CTA, on a batched plan of
Gaussian mixtures (GAUSSIAN, the distance in the dot form) and on a uniform
2-D cloud (MATERN32, the coordinate form), with 1, 8 and 32 right-hand
sides."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err, uniform_cloud
from fmca_gb300 import CovarianceKernel, H2Matrix
from test_batch import mixture_clouds


def _force_packed(H, R):
    cfg = H.tuned_config(R)
    cfg.update(near_halves=1, near_pack=1, near_persist=0, small_r_tensor=1)
    H.set_tuned_config(R, cfg)  # refused if the plan has no packed groups
    assert H.tuned_config(R)["near_pack"] == 1


@pytest.mark.gpu
@pytest.mark.parametrize("R", [1, 8, 32])
def test_packed_near_field_batched_mixtures(cuda_device, R):
    import torch
    clouds = mixture_clouds(6, seed=11, nmin=2000, nmax=20000)
    B = H2Matrix.batched(CovarianceKernel("GAUSSIAN", 0.2), clouds, 3, 0.8, precision="mixed")
    X = np.random.default_rng(R).standard_normal((B.rows(), R))
    x = torch.tensor(X, device=cuda_device)
    y1 = B.matvec(x).cpu().numpy()  # one leaf per CTA
    _force_packed(B, R)
    y2 = B.matvec(x).cpu().numpy()
    B.check_device_error()
    for i, P in enumerate(clouds):
        o, e = B.offsets[i], B.offsets[i + 1]
        Yi, _ = oracle.OraclePlan(P, None, 3, 0.8, 0).action(3, 0.2, X[o:e])
        assert rel_err(y2[o:e], Yi) < 1e-5, i
    assert rel_err(y2, y1) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("R", [8, 32])
def test_packed_near_field_uniform_2d(cuda_device, R):
    import torch
    P = uniform_cloud(30000, 2, seed=12)
    X = np.random.default_rng(R).standard_normal((P.shape[1], R))
    H = H2Matrix(CovarianceKernel("MATERN32", 0.3), P, P, 3, 0.8, precision="mixed")
    x = torch.tensor(X, device=cuda_device)
    y1 = H.matvec(x).cpu().numpy()
    _force_packed(H, R)
    y2 = H.matvec(x).cpu().numpy()
    H.check_device_error()
    Y_ref, _ = oracle.OraclePlan(P, None, 3, 0.8, 0).action(1, 0.3, X)
    assert rel_err(y2, Y_ref) < 1e-5
    assert rel_err(y2, y1) < 1e-5
