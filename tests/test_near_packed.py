"""Near field of the tensor-core kernel sum on packed groups: the rows of up
to two consecutive row leaves per CTA (128 targets, one half) over the union
of the leaves' source intervals, every target masked to its own leaf's
sources (H2MatrixBase.h:143-146: the dense blocks of one row leaf).

CPU: the packed groups of batched and uniform plans (fmca_plan_near_packed)
cover every row once, a group's rows belong to one leaf or to two
consecutive ones, and the intervals that serve each leaf are exactly that
leaf's dense-block sources; plans where packing saves too little have none.
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


def _leaf_sources(H):
    """row leaf cluster -> sorted array of its dense blocks' source points
    (cluster order), and the leaf clusters sorted by first row."""
    meta, _ = H.clusters(0)
    cmeta, _ = H.clusters(1)
    r, c = H.blocks(1)
    src = {}
    for rr, cc in zip(r.tolist(), c.tolist()):
        b, n = int(cmeta[cc, 0]), int(cmeta[cc, 1])
        src.setdefault(rr, []).append(np.arange(b, b + n))
    src = {k: np.sort(np.concatenate(v)) for k, v in src.items()}
    leaves = sorted(src, key=lambda k: int(meta[k, 0]))
    return meta, src, leaves


def _check_packed(H):
    groups, ivl = H.near_packed()
    meta, src, leaves = _leaf_sources(H)
    n = H.rows()
    owner = np.full(n, -1, dtype=np.int64)
    for k in leaves:
        owner[int(meta[k, 0]):int(meta[k, 0] + meta[k, 1])] = k
    assert (owner >= 0).all()
    seen = np.zeros(n, dtype=np.int64)
    two = 0
    for tb, tc, ib, ie, sp in groups.tolist():
        assert 1 <= tc <= 128 and 1 <= sp <= tc and ib <= ie
        seen[tb:tb + tc] += 1
        la = owner[tb]
        assert (owner[tb:tb + sp] == la).all()
        parts = [np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int64)]
        for b, e, m in ivl[ib:ie].tolist():
            assert b < e and m in (1, 2, 3)
            for bit in (0, 1):
                if m >> bit & 1:
                    parts[bit] = np.concatenate([parts[bit], np.arange(b, e)])
        assert np.array_equal(np.sort(parts[0]), src[la])
        if sp < tc:
            two += 1
            lb = owner[tb + sp]
            assert lb != la and (owner[tb + sp:tb + tc] == lb).all()
            # consecutive leaves: the first leaf's rows end where the second's begin
            assert int(meta[la, 0] + meta[la, 1]) == int(meta[lb, 0])
            assert np.array_equal(np.sort(parts[1]), src[lb])
        else:
            assert parts[1].size == 0
    assert (seen == 1).all()
    return len(groups), two, len(leaves)


def test_packed_groups_of_batched_mixtures():
    clouds = mixture_clouds(8, seed=13, nmin=2000, nmax=20000)
    B = H2Matrix.batched(CovarianceKernel("GAUSSIAN", 0.2), clouds, 3, 0.8)
    ng, two, nleaves = _check_packed(B)
    assert two > 0 and ng * 10 <= nleaves * 9
    # no group holds rows of two clouds
    groups, _ = B.near_packed()
    off = np.asarray(B.offsets)
    for tb, tc, _, _, _ in groups.tolist():
        assert np.searchsorted(off, tb, "right") == np.searchsorted(off, tb + tc - 1, "right")


def test_packed_groups_of_uniform_clouds():
    # 2-D, p = 3: leaves of about 20 points, most groups hold two of them
    P = uniform_cloud(20000, 2, seed=14)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.3), P, P, 3, 0.8)
    ng, two, nleaves = _check_packed(H)
    assert two > 0 and ng * 10 <= nleaves * 9
    # 3-D, p = 3: leaves of 64..127 points fill most of 128 rows; packing
    # would save less than a tenth of the groups, so there are none
    P = uniform_cloud(30000, 3, seed=15)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.3), P, P, 3, 0.8)
    groups, ivl = H.near_packed()
    assert groups.shape == (0, 5) and ivl.shape == (0, 3)


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
