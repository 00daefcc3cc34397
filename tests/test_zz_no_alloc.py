"""fmca_matvec_static_scratch: the matvec for callers that cannot allocate
device memory on their working path (an application that owns all GPU
memory through its own allocator, or a loop that cannot afford the device
synchronisation of cudaMalloc / cudaFree).  It runs the same product as
fmca_matvec with its scratch in a fixed 64 MiB device array of the library.

Called here through the C ABI and compared with fmca_matvec, within the
tolerances of the other GPU tests, on two calls in a row.  Around the second
call (the first one looked up the array's device address) the GPU's free
memory and the plan's own device memory must stay exactly the same: the
call allocates nothing, neither itself nor through the plan's workspace.  This file is
collected last so that a run stopping at its first failure has run every
other test already; it also passes on its own in a fresh process."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err, uniform_cloud
from fmca_gb300 import CovarianceKernel, H2Matrix, _lib

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-5, "mixed": 1e-5}
PREC = {"fp64": _lib.PREC_FP64, "fp32": _lib.PREC_FP32, "mixed": _lib.PREC_MIXED}


def static_matvec(H, cov, prec, x, y, stream):
    d = cov.desc()
    dt = _lib.DTYPE_F64 if x.dtype.is_floating_point and x.element_size() == 8 else _lib.DTYPE_F32
    return _lib.load().fmca_matvec_static_scratch(
        H.handle, C.byref(d), PREC[prec], dt, _lib.ORDER_NATURAL, x.shape[1],
        C.c_void_p(x.data_ptr()), x.stride(0), x.stride(1),
        C.c_void_p(y.data_ptr()), y.stride(0), y.stride(1), C.c_void_p(stream.cuda_stream))


def plan_device_bytes(H):
    n = C.c_size_t(0)
    assert _lib.load().fmca_plan_device_bytes(H.handle, C.byref(n)) == _lib.FMCA_OK
    return n.value


@pytest.mark.parametrize("prec", ["fp64", "fp32", "mixed"])
def test_static_scratch_matches_matvec(cuda_device, prec):
    import torch
    P = uniform_cloud(6000, 3, seed=41)
    X = np.random.default_rng(41).standard_normal((6000, 24))
    cov = CovarianceKernel("MATERN32", 0.4)
    H = H2Matrix(cov, P, P, 3, 0.8)
    x = torch.tensor(X, device=cuda_device)
    y_ref = H.matvec(x, precision=prec)          # fmca_matvec; makes the plan resident
    stream = torch.cuda.current_stream(cuda_device)
    for call in range(2):                          # two calls in a row share the scratch
        y = torch.full_like(y_ref, float("nan"))
        torch.cuda.synchronize(cuda_device)
        free0, held0 = torch.cuda.mem_get_info(cuda_device)[0], plan_device_bytes(H)
        assert static_matvec(H, cov, prec, x, y, stream) == _lib.FMCA_OK
        torch.cuda.synchronize(cuda_device)
        if call == 1:
            assert torch.cuda.mem_get_info(cuda_device)[0] == free0
            assert plan_device_bytes(H) == held0
        assert torch.isfinite(y).all()
        assert rel_err(y.cpu().numpy(), y_ref.cpu().numpy()) < TOL[prec]
    H.check_device_error()


def test_static_scratch_rejects_oversized_and_non_resident(cuda_device):
    import torch
    stream = torch.cuda.current_stream(cuda_device)
    cov = CovarianceKernel("EXPONENTIAL", 1.0)
    # scratch beyond the 64 MiB maximum
    P = uniform_cloud(200000, 3, seed=3)
    H = H2Matrix(cov, P, P, 2, 0.8)
    assert H.workspace_bytes(64, "fp64") > 64 << 20
    x = torch.zeros((200000, 64), dtype=torch.float64, device=cuda_device)
    y = torch.empty_like(x)
    st = static_matvec(H, cov, "fp64", x, y, stream)
    assert st == 2  # FMCA_ERR_UNSUPPORTED
    assert b"static scratch" in _lib.load().fmca_last_error()
    # a plan that never ran a matvec on this device is not resident
    P2 = uniform_cloud(2000, 3, seed=4)
    H2 = H2Matrix(cov, P2, P2, 2, 0.8)
    x2 = torch.zeros((2000, 4), dtype=torch.float64, device=cuda_device)
    y2 = torch.empty_like(x2)
    assert static_matvec(H2, cov, "fp64", x2, y2, stream) == 1  # FMCA_ERR_INVALID_ARGUMENT
    assert b"resident" in _lib.load().fmca_last_error()
