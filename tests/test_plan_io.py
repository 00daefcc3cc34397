"""Plan files (fmca_plan_save / fmca_plan_load): a loaded plan equals the
saved one (trees, permutations, block lists, statistics, interpolation
nodes), the file is a sequence of matrices in the binary layout of FMCA's
print2bin (FMCA/src/util/IO.h:532-580), and malformed files are refused."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err, sphere_cloud, uniform_cloud
from fmca_gb300 import CovarianceKernel, FmcaError, H2Matrix, _lib

ERR = {v: k for k, v in _lib.STATUS_NAMES.items()}


def same_plan(A, B):
    assert A.info == B.info
    for side in (0, 1):
        ma, ba = A.clusters(side)
        mb, bb = B.clusters(side)
        assert np.array_equal(ma, mb) and np.array_equal(ba, bb)
    assert np.array_equal(A.rindices(), B.rindices())
    assert np.array_equal(A.cindices(), B.cindices())
    for kind in (0, 1):
        ra, ca = A.blocks(kind)
        rb, cb = B.blocks(kind)
        assert np.array_equal(ra, rb) and np.array_equal(ca, cb)
    assert np.array_equal(A.statistics(False), B.statistics(False))
    na, ia = A.interpolation_nodes()
    nb, ib = B.interpolation_nodes()
    assert np.array_equal(na, nb)
    assert (ia is None and ib is None) or np.array_equal(ia, ib)


def read_print2bin(path):
    """The file as a list of (element size, rows, cols, raw bytes) records,
    read the way bin2Mat reads one matrix (IO.h:585-626)."""
    raw = open(path, "rb").read()
    out, pos = [], 0
    while pos < len(raw):
        size, rowmajor, rows, cols = np.frombuffer(raw, dtype=np.uint64, count=4, offset=pos)
        pos += 32
        assert rowmajor == 0
        nbytes = int(size * rows * cols)
        out.append((int(size), int(rows), int(cols), raw[pos:pos + nbytes]))
        pos += nbytes
    assert pos == len(raw)
    return out


CASES = {
    "tensor": lambda: (uniform_cloud(6000, 3, seed=1), None, 3, "tensor"),
    "total_degree": lambda: (uniform_cloud(6000, 3, seed=2), None, 4, "total_degree"),
    "unsymmetric": lambda: (sphere_cloud(5000, seed=3), sphere_cloud(3000, seed=4), 3, "tensor"),
    "two_dim": lambda: (uniform_cloud(4000, 2, seed=5), None, 5, "total_degree"),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_round_trip(tmp_path, case):
    Pr, Pc, p, interp = CASES[case]()
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), Pr, Pr if Pc is None else Pc, p, 0.8,
                 min_leaf=32, interpolator=interp)
    f = tmp_path / "plan.bin"
    H.save(f)
    G = H2Matrix.load(f, CovarianceKernel("MATERN32", 0.5))
    same_plan(H, G)
    assert G.interpolator == interp and G.p == p
    assert np.array_equal(G.offsets, [0, Pr.shape[1]])
    recs = read_print2bin(f)
    head = np.frombuffer(recs[0][3], dtype=np.int64)
    assert recs[0][:3] == (8, 16, 1) and head[0] == 0x464D4341 and head[2] == Pr.shape[0]
    assert recs[1][:3] == (8, 1, 1) and np.frombuffer(recs[1][3])[0] == 0.8
    pts = np.frombuffer(recs[2][3]).reshape(recs[2][2], recs[2][1]).T
    assert recs[2][1] == Pr.shape[0] and np.array_equal(pts, Pr)


def test_batched_round_trip(tmp_path):
    rng = np.random.default_rng(6)
    clouds = [rng.random((3, n)) for n in (700, 2500, 1300)]
    H = H2Matrix.batched(CovarianceKernel("GAUSSIAN", 0.2), clouds, p=3, eta=0.8)
    f = tmp_path / "batch.bin"
    H.save(f)
    G = H2Matrix.load(f, CovarianceKernel("GAUSSIAN", 0.2))
    same_plan(H, G)
    assert np.array_equal(G.offsets, [0, 700, 3200, 4500])
    assert np.array_equal(H.cloud_offsets(), H.offsets)


def test_malformed_files_are_refused(tmp_path):
    P = uniform_cloud(3000, 3, seed=7)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 3, 0.8)
    f = tmp_path / "plan.bin"
    H.save(f)
    raw = bytearray(open(f, "rb").read())

    def refused(data):
        g = tmp_path / "bad.bin"
        g.write_bytes(bytes(data))
        with pytest.raises(FmcaError) as e:
            H2Matrix.load(g, CovarianceKernel("MATERN32", 0.5))
        assert e.value.status == ERR["FMCA_ERR_INVALID_ARGUMENT"]

    refused(raw[:len(raw) // 2])                # truncated
    bad = bytearray(raw)
    bad[32] ^= 0xFF                              # magic of the header
    refused(bad)
    recs = read_print2bin(f)
    # first entry of the row permutation: an index out of range
    off = sum(32 + len(r[3]) for r in recs[:4]) + 32
    bad = bytearray(raw)
    bad[off:off + 4] = np.uint32(10**8).tobytes()
    refused(bad)
    with pytest.raises(FmcaError):
        H2Matrix.load(tmp_path / "missing.bin", CovarianceKernel("MATERN32", 0.5))


# record index of every matrix in a plan file of one cloud: header, eta, the
# two point clouds, the two trees (11 records each), then the block lists,
# leaves, transfer data, nodes and cloud offsets
ROW_TREE = dict(zip(["perm", "begin", "size", "level", "parent", "son0", "nsons", "bbmin",
                     "bbmax", "bbext", "level_ptr"], range(4, 15)))
LISTS = dict(zip(["far_row", "far_col", "near_row", "near_col", "far_ptr", "far_idx",
                  "near_ptr", "near_ivl", "row_leaves", "col_leaves", "row_E", "col_E",
                  "row_nodes", "col_nodes", "cloud_offsets"], range(26, 41)))
DTYPES = {"perm": np.uint32, "begin": np.uint32, "size": np.uint32, "near_ivl": np.uint32,
          "row_E": np.float64, "col_E": np.float64, "cloud_offsets": np.int64}


def write_print2bin(path, recs):
    with open(path, "wb") as f:
        for size, rows, cols, data in recs:
            f.write(np.array([size, 0, rows, cols], dtype=np.uint64).tobytes())
            f.write(data)


def corrupted(recs, field, edit):
    """recs with the array of `field` replaced by edit(copy of the array)."""
    k = ROW_TREE.get(field, LISTS.get(field))
    dt = DTYPES.get(field, np.int32)
    a = edit(np.frombuffer(recs[k][3], dtype=dt).copy())
    out = list(recs)
    out[k] = (np.dtype(dt).itemsize, a.size, 1, a.astype(dt).tobytes())
    return out


def test_corrupted_structure_fields_are_refused(tmp_path):
    """Every structural array of a plan file is checked before it reaches the
    device: levels, parents, sons, level offsets, CSR offsets, intervals,
    leaves, transfer data sizes and cloud offsets."""
    P = uniform_cloud(3000, 3, seed=7)
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 3, 0.8)
    f = tmp_path / "plan.bin"
    H.save(f)
    recs = read_print2bin(f)
    C = H.info["row_clusters"]

    def setv(i, v):
        def e(a):
            a[i] = v
            return a
        return e

    def swap_first_interval(a):
        a[0] = a[1] + 1
        return a

    cases = {
        "perm": lambda a: setv(1, a[0])(a),             # an index twice
        "level": setv(5, 99),                            # level past the last one
        "parent": setv(3, C + 7),                        # parent out of range
        "son0": setv(0, C - 1),                          # sons past the last cluster
        "nsons": setv(0, 10**6),
        "level_ptr": setv(1, 10**6),                     # offsets not monotone
        "far_ptr": setv(0, 1),                           # CSR not starting at 0
        "near_ptr": setv(1, -1),                         # CSR not monotone
        "near_ivl": swap_first_interval,                 # interval with begin > end
        "row_leaves": setv(0, 0),                        # the root as a leaf
        "row_E": lambda a: a[:-1],                       # transfer data one short
        "cloud_offsets": lambda a: np.array([0, 5], dtype=np.int64),
    }
    for field, edit in cases.items():
        g = tmp_path / f"bad_{field}.bin"
        write_print2bin(g, corrupted(recs, field, edit))
        with pytest.raises(FmcaError) as e:
            H2Matrix.load(g, CovarianceKernel("MATERN32", 0.5))
        assert e.value.status == ERR["FMCA_ERR_INVALID_ARGUMENT"], field
    # the untouched records still load
    g = tmp_path / "same.bin"
    write_print2bin(g, recs)
    same_plan(H, H2Matrix.load(g, CovarianceKernel("MATERN32", 0.5)))


@pytest.mark.gpu
@pytest.mark.parametrize("interp", ["tensor", "total_degree"])
def test_loaded_plan_gives_the_same_product(cuda_device, tmp_path, interp):
    P = uniform_cloud(20000, 3, seed=8)
    x = np.random.default_rng(8).standard_normal((20000, 4))
    H = H2Matrix(CovarianceKernel("MATERN32", 0.5), P, P, 4, 0.8, min_leaf=64,
                 precision="fp64", interpolator=interp)
    f = tmp_path / "plan.bin"
    H.save(f)
    G = H2Matrix.load(f, CovarianceKernel("MATERN32", 0.5), precision="fp64")
    assert rel_err(G.action(x), H.action(x)) <= 1e-14
