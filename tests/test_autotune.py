"""The autotuner (fmca_plan_set_autotune / fmca_plan_tuned_config).

With the autotuner on, the first mixed-precision matvec of a (precision,
kernel, right-hand sides) key measures the launch shapes of the kernel sums
and the transfer passes with CUDA events and keeps the fastest; later calls
of that key reuse them without tuning again.  The tests check the cache
(one tuning per key, none for another plan until it tunes itself), that the
chosen shapes lie in the tuned ranges, and that tuned products equal the
default-shape products and the FP64 oracle within the mixed-precision
tolerance (1e-5), for 32 right-hand sides on a 3-D degree-4 plan (paired
tensor-grid far field) and 8 right-hand sides on a 2-D plan (the choice
between CUDA cores and padded tensor cores)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err, uniform_cloud
from fmca_gb300 import CovarianceKernel, H2Matrix

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,p,R,kname,kt", [(3, 4, 32, "MATERN32", 1), (2, 5, 8, "EXPONENTIAL", 0)])
def test_tuned_shapes_are_cached_and_give_the_same_product(cuda_device, dim, p, R, kname, kt):
    import torch
    n = 30000
    P = uniform_cloud(n, dim, seed=21)
    X = np.random.default_rng(21).standard_normal((n, R))
    cov = CovarianceKernel(kname, 0.3)
    Y_ref, _ = oracle.OraclePlan(P, None, p, 0.8, 64).action(kt, 0.3, X)
    x = torch.tensor(X, device=cuda_device)
    D = H2Matrix(cov, P, P, p, 0.8, min_leaf=64, precision="mixed")
    y_default = D.matvec(x).cpu().numpy()
    assert D.tuned_config(R)["tuned"] == 0
    H = H2Matrix(cov, P, P, p, 0.8, min_leaf=64, precision="mixed")
    H.set_autotune(True)
    ys = []
    for _ in range(3):
        ys.append(H.matvec(x).cpu().numpy())
        H.check_device_error()
    cfg = H.tuned_config(R)
    assert cfg["tuned"] == 1 and cfg["tunings"] == 1, cfg
    assert 4 <= cfg["near_stages"] <= 7 and 1 <= cfg["near_unit"] <= 3
    assert 4 <= cfg["far_grid_stages"] <= 7 and 1 <= cfg["far_grid_unit"] <= 3
    assert 5 <= cfg["far_node_stages"] <= 7 and 1 <= cfg["far_node_unit"] <= 3
    assert cfg["small_r_tensor"] in (0, 1) and cfg["tune_us"] > 0
    for y in ys:
        assert rel_err(y, Y_ref) < 1e-5
        assert rel_err(y, y_default) < 1e-5
    # the tuned calls of one key agree with each other to rounding
    assert rel_err(ys[2], ys[1]) < 1e-6
    # another key tunes once more; the first key's entry stays
    H.matvec(x[:, :R - 1].contiguous())
    assert H.tuned_config(R - 1)["tunings"] == 2
    assert H.tuned_config(R) == {**cfg, "tunings": 2}
    # the defaults of an untuned plan are unaffected
    assert D.tuned_config(R)["tuned"] == 0
