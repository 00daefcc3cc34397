"""Property tests over random small clouds (hypothesis; CPU only): the plan
builder against the oracle and the H2 invariants the reference relies on.

For random clouds (n 1..400, dim 1..3, clustered or uniform, some coordinates
tied), degrees 1..5, eta 0.1..1.0, minimum leaf 1..50 and the four kernels of
the reference's tests (EXPONENTIAL, MATERN32, MATERN52, GAUSSIAN):
- the product's plan and the oracle build the same permutation, cluster
  boxes and block lists (ClusterTreeInitializer_ClusterTree.h:24-132,
  H2MatrixBase.h:160-191);
- the far and near blocks tile K exactly once: every (row point, column
  point) pair lies in one block;
- the transfer identity < 1e-13 (compute_cluster_bases_impl.h:66-76) holds
  for both interpolators;
- with eta = 0 no block is admissible and the H2 product is the dense
  product;
- total degree: the plan's DeMarchi nodes equal the oracle's;
- a plan written to a file and read back is the same plan."""
from __future__ import annotations

import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import HealthCheck, given, settings  # noqa: E402
from hypothesis import strategies as st  # noqa: E402

import oracle  # noqa: E402
from conftest import rel_err  # noqa: E402
from fmca_gb300 import CovarianceKernel, H2Matrix  # noqa: E402

KERNELS = ["EXPONENTIAL", "MATERN32", "MATERN52", "GAUSSIAN"]
SETTINGS = dict(max_examples=150, deadline=None,
                suppress_health_check=[HealthCheck.too_slow])


@st.composite
def clouds(draw, max_n=400):
    dim = draw(st.integers(1, 3))
    n = draw(st.integers(1, max_n))
    seed = draw(st.integers(0, 2**31 - 1))
    kind = draw(st.sampled_from(["uniform", "clusters", "ties"]))
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        P = rng.random((dim, n))
    elif kind == "clusters":
        centres = rng.random((dim, 4))
        P = centres[:, rng.integers(0, 4, n)] + 0.02 * rng.standard_normal((dim, n))
    else:
        P = np.floor(rng.random((dim, n)) * 8) / 8
    return np.asfortranarray(P)


def block_cover(meta, far, near, n):
    """For every (row, col) point pair in cluster order, the number of blocks
    that contain it (meta: begin and size per cluster, both sides the same
    tree)."""
    cover = np.zeros((n, n), dtype=np.int32)
    for rows, cols in (far, near):
        for r, c in zip(rows, cols):
            cover[meta[r, 0]:meta[r, 0] + meta[r, 1], meta[c, 0]:meta[c, 0] + meta[c, 1]] += 1
    return cover


@given(P=clouds(), p=st.integers(1, 5), eta=st.floats(0.1, 1.0),
       leaf=st.integers(1, 50))
@settings(**SETTINGS)
def test_plan_equals_oracle_and_blocks_tile_once(P, p, eta, leaf):
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, p, eta, min_leaf=leaf)
    O = oracle.OraclePlan(P, None, p, eta, leaf)
    assert np.array_equal(H.rindices(), O.perm(0))
    mh, bh = H.clusters(0)
    mo, bo = O.clusters(0)
    assert np.array_equal(mh, mo) and np.array_equal(bh, bo)
    far, near = H.blocks(0), H.blocks(1)
    assert sorted(zip(*far)) == sorted(zip(*O.blocks(0)))
    assert sorted(zip(*near)) == sorted(zip(*O.blocks(1)))
    n = P.shape[1]
    if n <= 200:
        assert (block_cover(mh, far, near, n) == 1).all()
    assert sorted(H.rindices().tolist()) == list(range(n))


@given(P=clouds(max_n=300), p=st.integers(1, 5), eta=st.floats(0.1, 1.0),
       leaf=st.integers(1, 50), td=st.booleans())
@settings(**SETTINGS)
def test_transfer_identity(P, p, eta, leaf, td):
    O = oracle.OraclePlan(P, None, p, eta, leaf,
                          interpolator="total_degree" if td else "tensor")
    assert O.check_transfer() < 1e-13


@given(P=clouds(max_n=250), p=st.integers(1, 4), kname=st.sampled_from(KERNELS),
       l=st.floats(0.1, 2.0), td=st.booleans())
@settings(**SETTINGS)
def test_no_admissible_blocks_is_dense(P, p, kname, l, td):
    ktype = KERNELS.index(kname)
    x = np.random.default_rng(P.shape[1]).standard_normal((P.shape[1], 2))
    O = oracle.OraclePlan(P, None, p, 0.0, 1, interpolator="total_degree" if td else "tensor")
    assert O.n_far == 0
    y, _ = O.action(ktype, l, x)
    yd = oracle.dense_matvec(ktype, l, P, P, x)
    assert rel_err(y, yd) < 1e-13


@given(dim=st.integers(1, 3), p=st.integers(1, 5), seed=st.integers(0, 1000))
@settings(max_examples=60, deadline=None)
def test_total_degree_nodes_equal_oracle(dim, p, seed):
    P = np.asfortranarray(np.random.default_rng(seed).random((dim, 50)))
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, p, 0.8,
                 interpolator="total_degree")
    O = oracle.OraclePlan(P, None, p, 0.8, interpolator="total_degree")
    n1, i1 = H.interpolation_nodes()
    n2, i2 = O.interp()
    assert np.array_equal(n1, n2)
    assert np.abs(i1 - i2).max() <= 1e-12 * np.abs(i2).max()


@given(P=clouds(max_n=300), p=st.integers(1, 4), eta=st.floats(0.1, 1.0),
       leaf=st.integers(1, 50), td=st.booleans())
@settings(max_examples=60, deadline=None)
def test_plan_file_round_trip(tmp_path_factory, P, p, eta, leaf, td):
    if td and P.shape[0] > 3:
        return
    interp = "total_degree" if td else "tensor"
    H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, p, eta, min_leaf=leaf,
                 interpolator=interp)
    f = tmp_path_factory.mktemp("plan") / "p.bin"
    H.save(f)
    G = H2Matrix.load(f, CovarianceKernel("EXPONENTIAL", 1.0))
    assert G.info == H.info
    assert np.array_equal(G.rindices(), H.rindices())
    mh, bh = H.clusters(0)
    mg, bg = G.clusters(0)
    assert np.array_equal(mh, mg) and np.array_equal(bh, bg)
    for kind in (0, 1):
        assert sorted(zip(*G.blocks(kind))) == sorted(zip(*H.blocks(kind)))
