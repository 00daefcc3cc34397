"""Cluster trees and block lists: the product's plan builder and the oracle
against the golden fixtures of an independent numpy restatement
(tests/golden/gen_structure.py), bit for bit."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from fmca_gb300 import CovarianceKernel, H2Matrix
from golden.gen_structure import cloud

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "structure.json")))


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def fingerprint_of(perm, meta, bb, far, near):
    far = np.array(sorted(zip(*far)), dtype=np.int32).reshape(-1, 2)
    near = np.array(sorted(zip(*near)), dtype=np.int32).reshape(-1, 2)
    return dict(perm_sha=sha(perm.astype(np.uint32)), meta_sha=sha(meta[:, :3].astype(np.int32)),
                bb_sha=sha(bb), far_sha=sha(far), near_sha=sha(near),
                far_blocks=len(far), near_blocks=len(near))


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_plan_matches_golden(name):
    g = GOLDEN[name]
    P = cloud(g["cloud"], g["n"], g["dim"])
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, g["degree"], g["eta"],
                 min_leaf=g["min_leaf"])
    meta, bb = H.clusters(0)
    fp = fingerprint_of(H.rindices(), meta, bb, H.blocks(0), H.blocks(1))
    for k, v in fp.items():
        assert v == g[k], k
    assert H.info["row_clusters"] == g["clusters"]
    assert H.info["near_pairs"] == g["near_pairs"]
    if "perm" in g:
        assert H.rindices().tolist() == g["perm"]


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_oracle_matches_golden(name):
    g = GOLDEN[name]
    P = cloud(g["cloud"], g["n"], g["dim"])
    O = oracle.OraclePlan(P, None, g["degree"], g["eta"], g["min_leaf"])
    meta, bb = O.clusters(0)
    fp = fingerprint_of(O.perm(0), meta, bb, O.blocks(0), O.blocks(1))
    for k, v in fp.items():
        assert v == g[k], k


def test_plan_equals_oracle_unsymmetric():
    rng = np.random.default_rng(3)
    Pr = rng.random((3, 3000)) * 2 - 1
    Pc = rng.random((3, 1700)) * 2 - 1
    H = H2Matrix(CovarianceKernel("GAUSSIAN", 0.3), Pr, Pc, 2, 0.7, min_leaf=20)
    O = oracle.OraclePlan(Pr, Pc, 2, 0.7, 20)
    assert np.array_equal(H.rindices(), O.perm(0))
    assert np.array_equal(H.cindices(), O.perm(1))
    for side in (0, 1):
        mh, bh = H.clusters(side)
        mo, bo = O.clusters(side)
        assert np.array_equal(mh, mo) and np.array_equal(bh, bo)
    for kind in (0, 1):
        assert sorted(zip(*H.blocks(kind))) == sorted(zip(*O.blocks(kind)))
    assert np.array_equal(H.statistics(False).ravel(), O.statistics())


@pytest.mark.parametrize("leaf", [0, 1, 7, 50, 300])
def test_permutation_complete(leaf):
    # tests/test_ClusterTree.cpp:50-57: every index appears exactly once
    P = np.random.default_rng(leaf).random((3, 5000))
    H = H2Matrix(CovarianceKernel("EXPONENTIAL"), P, P, 1, 0.8, min_leaf=leaf)
    perm = H.rindices()
    assert np.array_equal(np.sort(perm), np.arange(5000))
    meta, _ = H.clusters(0)
    # children partition their father's index range
    for c in range(1, meta.shape[0]):
        f = meta[c, 3]
        assert meta[f, 0] <= meta[c, 0] and meta[c, 0] + meta[c, 1] <= meta[f, 0] + meta[f, 1]


def test_statistics_like_reference():
    P = cloud("uniform", 10000, 3)
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, 3, 0.8, min_leaf=64)
    st = H.statistics(False).ravel()
    O = oracle.OraclePlan(P, None, 3, 0.8, 64)
    assert np.array_equal(st, O.statistics())
    assert st[0] == 10000 and st[1] == 10000
    assert st[2] == GOLDEN["c1"]["far_blocks"] and st[3] == GOLDEN["c1"]["near_blocks"]


def test_degenerate_clouds():
    # duplicated points and a flat dimension: the flat-box fix and ties
    rng = np.random.default_rng(1)
    P = rng.random((3, 1000))
    P[2] = 0.5
    P[:, 500:] = P[:, :500]
    H = H2Matrix(CovarianceKernel("MATERN32", 0.4), P, P, 2, 0.8, min_leaf=8)
    O = oracle.OraclePlan(P, None, 2, 0.8, 8)
    assert np.array_equal(H.rindices(), O.perm(0))
    mh, bh = H.clusters(0)
    mo, bo = O.clusters(0)
    assert np.array_equal(bh, bo)
    assert sorted(zip(*H.blocks(0))) == sorted(zip(*O.blocks(0)))
    assert sorted(zip(*H.blocks(1))) == sorted(zip(*O.blocks(1)))


def test_single_point_and_tiny():
    for n in (1, 2, 5):
        P = np.random.default_rng(n).random((3, n))
        H = H2Matrix(CovarianceKernel("EXPONENTIAL"), P, P, 2, 0.8)
        assert H.info["row_clusters"] == 1
        assert H.info["far_blocks"] == 0 and H.info["near_blocks"] == 1


@pytest.mark.parametrize("dim", [2, 3])
def test_parallel_tree_build_equals_oracle(dim):
    # clouds large enough that the plan splits the clusters of a level on
    # several host threads (from 65,536 points per level), with a third of
    # the coordinates quantised so that the sorts meet ties; the oracle
    # builds the same tree by the reference's serial depth-first recursion
    rng = np.random.default_rng(40 + dim)
    P = rng.random((dim, 150000))
    P[:, ::3] = np.floor(P[:, ::3] * 32) / 32
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, 2, 0.8, min_leaf=32)
    O = oracle.OraclePlan(P, None, 2, 0.8, 32)
    assert np.array_equal(H.rindices(), O.perm(0))
    mh, bh = H.clusters(0)
    mo, bo = O.clusters(0)
    assert np.array_equal(mh, mo) and np.array_equal(bh, bo)
    for kind in (0, 1):
        assert sorted(zip(*H.blocks(kind))) == sorted(zip(*O.blocks(kind)))
