"""Bounded waits running out on the GPU, without a fault.

Every wait of the kernel sums (near and far field, tensor-core and CUDA-core
versions) is bounded.  For one matvec the test shortens that bound to 1 ms
(fmca_plan_set_wait_limit) and turns on the stalled-wait hook
(fmca_plan_set_stalled_wait): the first wait of every kernel-sum CTA is then
on a barrier that nothing completes.  The kernels raise the plan's error
flag, drain their own copies and products under their fixed drain limit,
free tensor memory and return.  The test checks that the host reads
FMCA_ERR_TIMEOUT from fmca_plan_check_device_error, and that the next
matvecs with the default limit, on the same plan and GPU context, again
equal the FP64 oracle."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err, uniform_cloud
from fmca_gb300 import CovarianceKernel, FmcaError, H2Matrix, _lib

ERR = {v: k for k, v in _lib.STATUS_NAMES.items()}


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["mixed", "fp32"])
def test_wait_limit_runs_out_and_the_context_stays_usable(cuda_device, prec):
    import torch
    n, R = 20000, 32
    P = uniform_cloud(n, 3, seed=5)
    X = np.random.default_rng(5).standard_normal((n, R))
    O = oracle.OraclePlan(P, None, 4, 0.8, 64)
    Y_ref, _ = O.action(1, 0.5, X)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 4, 0.8, min_leaf=64, precision=prec)
    x = torch.tensor(X, device=cuda_device)
    H.matvec(x)
    H.check_device_error()
    H.set_wait_limit(1_000_000)
    H.set_stalled_wait(True)
    H.matvec(x)
    with pytest.raises(FmcaError) as e:
        H.check_device_error()
    assert e.value.status == ERR["FMCA_ERR_TIMEOUT"]
    H.check_device_error()  # the flag was cleared
    H.set_stalled_wait(False)
    H.set_wait_limit(0)
    for _ in range(2):
        Y = H.matvec(x)
        H.check_device_error()
        assert rel_err(Y.cpu().numpy(), Y_ref) < 1e-5
