"""Many independent point clouds in one plan (block-diagonal H2 matrix) and
matvecs recorded into CUDA graphs.

CPU: the batched plan holds every cloud's own tree and block lists, offset.
GPU: one batched matvec (all clouds per launch) against the oracle run cloud
by cloud, in every precision; a graph replay against the direct call; the
persistent kernel sums (one CTA per SM over the groups of every cloud) in a
graph against the oracle."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import rel_err
from fmca_gb300 import CovarianceKernel, H2Matrix

TOL = {"fp64": 1e-12, "fp32": 1e-5, "mixed": 1e-5}


def mixture_clouds(count, seed=0, nmin=300, nmax=5000):
    """Clouds of log-uniform size from a 3-D Gaussian mixture (8 components,
    sigma = 0.05, centres uniform in [0,1]^3)."""
    rng = np.random.default_rng(seed)
    centres = rng.random((8, 3))
    out = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        comp = rng.integers(0, 8, n)
        out.append((centres[comp] + 0.05 * rng.standard_normal((n, 3))).T.copy())
    return out


def test_batched_plan_is_union_of_single_plans():
    clouds = mixture_clouds(5, seed=1)
    cov = CovarianceKernel("GAUSSIAN", 0.2)
    B = H2Matrix.batched(cov, clouds, 3, 0.8)
    singles = [H2Matrix(cov, P, P, 3, 0.8) for P in clouds]
    assert B.info["n_rows"] == sum(P.shape[1] for P in clouds)
    assert B.info["far_blocks"] == sum(S.info["far_blocks"] for S in singles)
    assert B.info["near_blocks"] == sum(S.info["near_blocks"] for S in singles)
    assert B.info["near_pairs"] == sum(S.info["near_pairs"] for S in singles)
    perm = B.rindices()
    meta, bb = B.clusters(0)
    co = 0
    for i, S in enumerate(singles):
        o = B.offsets[i]
        n = clouds[i].shape[1]
        assert np.array_equal(perm[o:o + n], S.rindices() + o)
        m1, b1 = S.clusters(0)
        C = m1.shape[0]
        assert np.array_equal(meta[co:co + C, 0], m1[:, 0] + o)
        assert np.array_equal(meta[co:co + C, 1:3], m1[:, 1:3])
        assert np.array_equal(bb[co:co + C], b1)
        co += C
    st = B.statistics(False).ravel()
    assert st[2] == B.info["far_blocks"] and st[3] == B.info["near_blocks"]


@pytest.mark.gpu
@pytest.mark.parametrize("prec,deg", [("fp64", 3), ("fp32", 3), ("mixed", 3), ("mixed", 4)])
def test_batched_matvec_against_oracle(cuda_device, prec, deg):
    # degree 4 in 3-D: the far field on tensor grids, sibling row clusters
    # paired per CTA inside a forest of one tree per cloud
    import torch
    clouds = mixture_clouds(6, seed=2)
    R = 20
    cov = CovarianceKernel("GAUSSIAN", 0.2)
    B = H2Matrix.batched(cov, clouds, deg, 0.8, precision=prec)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((B.rows(), R))
    Y = B.matvec(torch.tensor(X, device=cuda_device)).cpu().numpy()
    for i, P in enumerate(clouds):
        o, e = B.offsets[i], B.offsets[i + 1]
        O = oracle.OraclePlan(P, None, deg, 0.8, 0)
        Yi, _ = O.action(3, 0.2, X[o:e])
        assert rel_err(Y[o:e], Yi) < TOL[prec], i
    B.check_device_error()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_graph_replay_matches_direct_call(cuda_device, prec):
    import torch
    clouds = mixture_clouds(4, seed=5)
    B = H2Matrix.batched(CovarianceKernel("MATERN32", 0.3), clouds, 3, 0.8, precision=prec)
    X = torch.tensor(np.random.default_rng(6).standard_normal((B.rows(), 32)),
                     device=cuda_device)
    ref = B.matvec(X)
    Y = torch.full_like(X, float("nan"))
    g = B.graph(X, Y)
    for _ in range(3):
        Y.fill_(float("nan"))
        g.launch()
        torch.cuda.synchronize()
        assert torch.equal(Y, ref)
    # the graph reads the bound x at every replay
    X.mul_(2.0)
    g.launch()
    torch.cuda.synchronize()
    assert rel_err(Y.cpu().numpy(), 2.0 * ref.cpu().numpy()) < TOL[prec]
    del g


@pytest.mark.gpu
def test_batched_adjoint_values(cuda_device):
    import torch
    clouds = mixture_clouds(3, seed=8, nmin=2000, nmax=4000)
    B = H2Matrix.batched(CovarianceKernel("MATERN52", 0.25), clouds, 3, 0.8, precision="fp64")
    rng = np.random.default_rng(9)
    X = rng.standard_normal((B.rows(), 2))
    Yv = rng.standard_normal((B.rows(), 2))
    out = B.adjoint(torch.tensor(X, device=cuda_device), torch.tensor(Yv, device=cuda_device))
    vals = out["values"].cpu().numpy()
    dX = out["dX"].cpu().numpy()
    ref = np.zeros(3)
    for i, P in enumerate(clouds):
        o, e = B.offsets[i], B.offsets[i + 1]
        O = oracle.OraclePlan(P, None, 3, 0.8, 0)
        v, d = oracle.adjoint(O, 2, 0.25, X[o:e], Yv[o:e])
        ref += v
        assert rel_err(dX[o:e], d) < 1e-10, i
    assert np.allclose(vals, ref, rtol=1e-10, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("deg", [3, 4])
def test_persistent_kernel_sums_over_all_clouds(cuda_device, deg):
    # one persistent launch per kernel sum: one CTA per SM runs the groups of
    # every cloud (the flattened near and far group lists) in turn, recorded
    # into a CUDA graph; against the oracle cloud by cloud
    import torch
    clouds = mixture_clouds(12, seed=10)
    R = 32
    cov = CovarianceKernel("GAUSSIAN", 0.2)
    B = H2Matrix.batched(cov, clouds, deg, 0.8, precision="mixed")
    X = torch.tensor(np.random.default_rng(11).standard_normal((B.rows(), R)), device=cuda_device)
    B.matvec(X)  # resident
    B.set_tuned_config(R, {**B.tuned_config(R), "near_persist": 1, "far_persist": 1})
    Y = torch.empty_like(X)
    g = B.graph(X, Y)
    for _ in range(2):
        g.launch()
        torch.cuda.synchronize()
        B.check_device_error()
        Yh, Xh = Y.cpu().numpy(), X.cpu().numpy()
        for i, P in enumerate(clouds):
            o, e = B.offsets[i], B.offsets[i + 1]
            Yi, _ = oracle.OraclePlan(P, None, deg, 0.8, 0).action(3, 0.2, Xh[o:e])
            assert rel_err(Yh[o:e], Yi) < TOL["mixed"], i
    del g
