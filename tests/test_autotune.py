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


SHAPES = [
    # near field with one target half (groups of up to 128 targets)
    dict(near_halves=1, near_stages=5, near_unit=1),
    dict(near_halves=1, near_stages=7, near_unit=2),
    # two halves at the ends of the tuned ranges
    dict(near_halves=2, near_stages=4, near_unit=3, far_grid_stages=4, far_grid_unit=3),
    dict(near_halves=2, near_stages=7, near_unit=1, far_grid_stages=6, far_grid_unit=1),
    # the far field on nodes instead of paired tensor grids
    dict(far_pairs=0, far_node_stages=7, far_node_unit=2),
    dict(far_pairs=0, far_node_stages=5, far_node_unit=1, wide_below=0, slice_below=0),
    # transfers: 8 warps and right-hand-side slices on every level
    dict(wide_below=1 << 30, slice_below=1 << 30),
    # persistent launches: one CTA per SM running the groups in turn
    dict(near_persist=1, far_persist=1),
    dict(near_persist=1, far_persist=1, near_halves=1, near_stages=6, near_unit=2,
         far_pairs=0, far_node_stages=6, far_node_unit=2),
    dict(near_persist=1, far_persist=1, near_stages=4, near_unit=3, far_grid_stages=4,
         far_grid_unit=3),
]


@pytest.mark.parametrize("leaf", [64, 200])
@pytest.mark.parametrize("shape", range(len(SHAPES)))
def test_set_shapes_match_the_oracle(cuda_device, shape, leaf):
    """Every launch shape the autotuner may choose (persistent launches
    included), set through fmca_plan_set_tuned_config, gives the FP64
    oracle's product within 1e-5
    (3-D, degree 4: paired tensor-grid far field available; leaves of 64..127
    and of 200..399 points, so one-half near groups hold one leaf or part of
    one)."""
    import torch
    n, R = 25000, 32
    P = uniform_cloud(n, 3, seed=22)
    X = np.random.default_rng(22).standard_normal((n, R))
    Y_ref, _ = oracle.OraclePlan(P, None, 4, 0.8, leaf).action(1, 0.45, X)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.45), P, P, 4, 0.8, min_leaf=leaf,
                 precision="mixed")
    x = torch.tensor(X, device=cuda_device)
    H.matvec(x)  # resident
    cfg = {**H.tuned_config(R), **SHAPES[shape]}
    H.set_tuned_config(R, cfg)
    got = H.tuned_config(R)
    assert got["tuned"] == 1 and all(got[k] == v for k, v in SHAPES[shape].items())
    for _ in range(2):
        y = H.matvec(x).cpu().numpy()
        H.check_device_error()
        assert rel_err(y, Y_ref) < 1e-5


def test_small_r_on_padded_tensor_cores(cuda_device):
    # 8 right-hand sides on the tensor cores (columns padded to 32)
    import torch
    n, R = 20000, 8
    P = uniform_cloud(n, 3, seed=23)
    X = np.random.default_rng(23).standard_normal((n, R))
    Y_ref, _ = oracle.OraclePlan(P, None, 3, 0.8, 64).action(3, 0.3, X)
    H = H2Matrix(CovarianceKernel("GAUSSIAN", 0.3), P, P, 3, 0.8, min_leaf=64, precision="mixed")
    x = torch.tensor(X, device=cuda_device)
    H.matvec(x)
    H.set_tuned_config(R, {**H.tuned_config(R), "small_r_tensor": 1, "near_halves": 1})
    y = H.matvec(x).cpu().numpy()
    H.check_device_error()
    assert rel_err(y, Y_ref) < 1e-5


def test_set_shapes_are_validated(cuda_device):
    import torch
    from fmca_gb300 import FmcaError
    P = uniform_cloud(3000, 3, seed=24)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 3, 0.8, precision="mixed")
    with pytest.raises(FmcaError):  # not resident yet
        H.set_tuned_config(32, H.tuned_config(32))
    H.matvec(torch.zeros((3000, 32), dtype=torch.float64, device=cuda_device))
    for bad in (dict(near_stages=8), dict(near_stages=2, near_unit=3), dict(near_halves=3),
                dict(far_pairs=2), dict(near_unit=0), dict(wide_below=-1),
                dict(near_persist=2), dict(far_persist=-1)):
        with pytest.raises(FmcaError):
            H.set_tuned_config(32, {**H.tuned_config(32), **bad})
    assert H.tuned_config(32)["tuned"] == 0
