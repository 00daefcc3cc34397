"""Plans built with a level sorter (Tree::build_with) and a block-pattern
builder, the path of fmca_plan_create_gpu.

CPU: h2_plan.cpp compiled with g++ together with a host level sorter that
sorts every segment with std::stable_sort (any sort gives the same order of
distinct keys) and reports equal neighbours like the GPU sorter.  On clouds
without equal coordinates the tree equals Tree::build's (permutation,
ranges, levels, links, boxes); with equal coordinates build_with refuses.

The pattern builder's ordering argument (leaves of a level-by-level
expansion sorted by their paths are in depth-first order) is restated on
the CPU against the host's block lists.

GPU: fmca_plan_create_gpu (one segmented radix sort per tree level, the block
tree level by level on the device) gives exactly the plan of
fmca_plan_create_ex (permutations,
clusters, block lists, statistics, nodes, products) on tie-free clouds, and
falls back to the host build, with the same plan, on clouds with equal
coordinates."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import rel_err, sphere_cloud, uniform_cloud

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "fmca_gb300", "csrc")

SRC = r"""
#include <algorithm>
#include <cstdio>
#include <vector>
#include "h2_plan.h"
using namespace fmca;
// the level sorter of the GPU path, restated on the host
struct HostSorter : LevelSorter {
  const double* P = nullptr;
  int dim = 0;
  std::vector<uint32_t> idx;
  int levels = 0;
  bool start(const double* P_, int dim_, uint32_t n) override {
    P = P_;
    dim = dim_;
    idx.resize(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    return true;
  }
  bool sort_level(const std::vector<SortSegment>& segs, std::vector<double>* cut,
                  bool* ties) override {
    ++levels;
    cut->resize(2 * segs.size());
    *ties = false;
    for (size_t s = 0; s < segs.size(); ++s) {
      const SortSegment g = segs[s];
      auto key = [&](uint32_t v) { return P[(size_t)v * dim + g.coord]; };
      std::stable_sort(idx.begin() + g.begin, idx.begin() + g.begin + g.size,
                       [&](uint32_t a, uint32_t b) { return key(a) < key(b); });
      for (uint32_t i = 1; i < g.size; ++i)
        if (key(idx[g.begin + i]) == key(idx[g.begin + i - 1])) *ties = true;
      (*cut)[2 * s] = key(idx[g.begin + g.size / 2 - 1]);
      (*cut)[2 * s + 1] = key(idx[g.begin + g.size / 2]);
    }
    return true;
  }
  bool finish(std::vector<uint32_t>* perm) override {
    *perm = idx;
    return true;
  }
};
// reads dim n min_csize and the points (dim x n); prints "same", "refused"
// or "different"
int main() {
  int dim;
  unsigned n, m;
  if (scanf("%d %u %u", &dim, &n, &m) != 3) return 2;
  std::vector<double> P((size_t)dim * n);
  for (auto& v : P)
    if (scanf("%lf", &v) != 1) return 2;
  Tree a, b;
  a.build(P.data(), dim, n, m, 3);
  HostSorter so;
  if (!b.build_with(&so, P.data(), dim, n, m)) {
    printf("refused %d\n", b.nclusters());
    return 0;
  }
  const bool same = a.perm == b.perm && a.begin == b.begin && a.size == b.size &&
                    a.level == b.level && a.parent == b.parent && a.son0 == b.son0 &&
                    a.nsons == b.nsons && a.bbmin == b.bbmin && a.bbmax == b.bbmax &&
                    a.bbext == b.bbext && a.level_ptr == b.level_ptr;
  printf("%s %d %d\n", same ? "same" : "different", a.nclusters(), so.levels);
  return 0;
}
"""


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("tree")
    src = d / "t.cpp"
    src.write_text(SRC)
    exe = d / "t"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", "-I", CSRC,
                    str(src), os.path.join(CSRC, "h2_plan.cpp"), "-o", str(exe)], check=True)
    return str(exe)


def run(prog, P, m):
    dim, n = P.shape
    inp = f"{dim} {n} {m}\n" + "\n".join(" ".join(repr(float(v)) for v in P[:, i])
                                        for i in range(n))
    out = subprocess.run([prog], input=inp, capture_output=True, text=True, check=True)
    return out.stdout.split()


@pytest.mark.parametrize("case", ["uniform3", "sphere", "aniso2", "line", "tiny", "odd"])
def test_level_sorter_tree_equals_host_tree(prog, case):
    rng = np.random.default_rng(abs(hash(case)) % 2**32)
    P = {"uniform3": lambda: uniform_cloud(20000, 3, seed=1),
         "sphere": lambda: sphere_cloud(9000, seed=2),
         "aniso2": lambda: uniform_cloud(12000, 2, seed=3) * np.array([[4.0], [1.0]]),
         "line": lambda: rng.random((1, 5000)),
         "tiny": lambda: rng.random((3, 5)),
         "odd": lambda: rng.standard_normal((3, 7777)) ** 3}[case]()
    res = run(prog, P, 32)
    assert res[0] == "same", res


def test_level_sorter_refuses_equal_coordinates(prog):
    # a lattice: every coordinate repeats, so std::sort's order of equal
    # keys decides the reference's permutation
    g = np.arange(12, dtype=np.float64)
    P = np.array(np.meshgrid(g, g, g, indexing="ij")).reshape(3, -1)
    assert run(prog, P, 16)[0] == "refused"


def test_path_keys_give_the_depth_first_order():
    """The ordering argument of the GPU pattern builder, restated on the CPU:
    expanding the block tree level by level and sorting its leaves by their
    left-aligned paths (two bits per level, the rank of a son pair in the
    order the reference's stack pops them) reproduces the raw block lists
    of the host's depth-first recursion exactly."""
    from fmca_gb300 import CovarianceKernel, H2Matrix
    for P, p, eta in ((uniform_cloud(6000, 3, seed=31), 3, 0.8),
                      (sphere_cloud(4000, seed=32), 2, 0.5),
                      (uniform_cloud(5000, 2, seed=33), 4, 1.2)):
        H = H2Matrix(CovarianceKernel("EXPONENTIAL", 1.0), P, P, p, eta)
        meta, bb = H.clusters(0)
        C, dim = meta.shape[0], P.shape[0]
        sons = [[] for _ in range(C)]
        for c in range(1, C):
            sons[meta[c, 3]].append(c)
        bmin, bmax, bext = bb[:, 0, :], bb[:, 1, :], bb[:, 2, :]

        def norm(v):
            s = v[0] * v[0]
            for k in range(1, len(v)):
                s = s + v[k] * v[k]
            return np.sqrt(s)
        rad = [0.5 * norm(bext[c]) for c in range(C)]
        qq = np.uint32(H.info["q"]) * np.uint32(H.info["q"])
        far, near, cur = [], [], [(0, 0, 0)]
        for depth in range(40):
            nxt = []
            for key, i, j in cur:
                v = [0.5 * (((bmin[i, d] - bmin[j, d]) + bmax[i, d]) - bmax[j, d])
                     for d in range(dim)]
                dist = max((norm(v) - rad[i]) - rad[j], 0.0)
                if max(rad[i], rad[j]) > eta * dist:
                    if not sons[i] or not sons[j]:
                        near.append((key, i, j))
                        continue
                    for b, sj in enumerate(sons[j]):
                        for a, si in enumerate(sons[i]):
                            rank = 3 - (2 * b + a)
                            nxt.append((key | (rank << (62 - 2 * depth)), si, sj))
                elif qq < np.uint32(meta[i, 1]) * np.uint32(meta[j, 1]):
                    far.append((key, i, j))
                else:
                    near.append((key, i, j))
            cur = nxt
            if not cur:
                break
        for kind, leaves in ((0, far), (1, near)):
            r, c = H.blocks(kind)
            leaves.sort()
            assert np.array_equal(r, [x[1] for x in leaves])
            assert np.array_equal(c, [x[2] for x in leaves])


# ---------------------------------------------------------------------------
# GPU: fmca_plan_create_gpu against fmca_plan_create_ex


def same_plans(A, B):
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


GPU_CASES = {
    "c2_like": lambda: (uniform_cloud(200000, 3, seed=11), None, 4, 128),
    "sphere": lambda: (sphere_cloud(60000, seed=12), None, 4, 96),
    "aniso2": lambda: (uniform_cloud(150000, 2, seed=13) * np.array([[4.0], [1.0]]), None, 5, 128),
    "two_clouds": lambda: (sphere_cloud(30000, seed=14), uniform_cloud(20000, 3, seed=15), 3, 0),
    "small": lambda: (uniform_cloud(300, 3, seed=16), None, 2, 0),
    "d1": lambda: (uniform_cloud(40000, 1, seed=17), None, 6, 0),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(GPU_CASES))
def test_gpu_built_plan_equals_host_plan(cuda_device, case):
    from fmca_gb300 import CovarianceKernel, H2Matrix
    Pr, Pc, p, leaf = GPU_CASES[case]()
    cov = CovarianceKernel("MATERN32", 0.5)
    Pc_ = Pr if Pc is None else Pc
    A = H2Matrix(cov, Pr, Pc_, p, 0.8, min_leaf=leaf, precision="fp64")
    B = H2Matrix(cov, Pr, Pc_, p, 0.8, min_leaf=leaf, precision="fp64", build="gpu")
    assert B.trees_on_gpu == (1 if Pc is None else 2) and B.pattern_on_gpu == 1
    same_plans(A, B)
    x = np.random.default_rng(1).standard_normal((Pc_.shape[1], 2))
    assert rel_err(B.action(x), A.action(x)) == 0.0


@pytest.mark.gpu
def test_gpu_build_falls_back_on_equal_coordinates(cuda_device):
    from fmca_gb300 import CovarianceKernel, H2Matrix
    g = np.arange(20, dtype=np.float64)
    P = np.array(np.meshgrid(g, g, g, indexing="ij")).reshape(3, -1) / 20.0
    cov = CovarianceKernel("EXPONENTIAL", 1.0)
    A = H2Matrix(cov, P, P, 3, 0.8, precision="fp64")
    B = H2Matrix(cov, P, P, 3, 0.8, precision="fp64", build="gpu")
    assert B.trees_on_gpu == 0 and B.pattern_on_gpu == 1
    same_plans(A, B)
