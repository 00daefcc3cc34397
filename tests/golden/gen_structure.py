"""Generates tests/golden/structure.json: cluster-tree and block-list
fingerprints from a pure numpy/Python restatement of FMCA's ClusterTree
(CardinalityBisection + shrinkToFit) and CompareCluster admissibility.

This restatement is independent of both the C++ plan builder and the C++
oracle; the fixture pins their tree, permutation and block lists.  Followed:
FMCA/src/Clustering/ClusterTreeInitializer_ClusterTree.h:24-132,
FMCA/src/Clustering/ClusterTreeSplitter.h:60-81,
FMCA/src/Clustering/Admissibility.h:19-29,95-115,
FMCA/src/H2Matrix/H2MatrixBase.h:160-191.

Run:  python tests/golden/gen_structure.py
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

EPS = np.finfo(float).eps
HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # name, n, dim, degree, min_leaf, eta, cloud
    ("small3d", 5000, 3, 2, 16, 0.8, "uniform"),
    ("c1", 10000, 3, 3, 64, 0.8, "uniform"),
    ("sphere", 20000, 3, 3, 64, 0.8, "sphere"),
    ("aniso2d", 20000, 2, 4, 32, 0.6, "aniso"),
    ("tiny", 300, 3, 1, 4, 0.5, "uniform"),
]


def cloud(kind, n, dim, seed=0):
    rng = np.random.default_rng(seed)
    if kind == "sphere":
        P = rng.standard_normal((3, n))
        return P / np.linalg.norm(P, axis=0)
    P = rng.random((dim, n))
    if kind == "aniso":
        P[0] *= 4
    return P


def build_tree(P, m):
    d, n = P.shape
    idx = np.arange(n)
    nodes = []  # dict(begin, size, level, sons, bb)
    lo = P.min(1).copy()
    hi = P.max(1).copy()
    lo -= EPS * np.abs(lo)
    hi += EPS * np.abs(hi)
    thr = 2 * m - 1 if m >= 1 else 1

    def rec(b, s, bb, lvl):
        me = len(nodes)
        nodes.append(dict(begin=b, size=s, level=lvl, sons=[], bb=None))
        if s > thr:
            ext = bb[:, 2]
            L = int(np.argmax(ext))  # first maximum
            seg = idx[b:b + s]
            idx[b:b + s] = seg[np.argsort(P[L, seg], kind="stable")]
            s1 = s // 2
            b1, b2 = bb.copy(), bb.copy()
            b1[L, 1] = P[L, idx[b + s1 - 1]]
            b1[L, 2] = b1[L, 1] - b1[L, 0]
            b2[L, 0] = P[L, idx[b + s1]]
            b2[L, 2] = b2[L, 1] - b2[L, 0]
            c1 = rec(b, s1, b1, lvl + 1)
            c2 = rec(b + s1, s - s1, b2, lvl + 1)
            nodes[me]["sons"] = [c1, c2]
        return me

    rec(0, n, np.stack([lo, hi, hi - lo], 1), 0)
    for k in range(len(nodes) - 1, -1, -1):  # sons have larger indices
        nd = nodes[k]
        if nd["sons"]:
            lo = np.minimum(nodes[nd["sons"][0]]["bb"][:, 0], nodes[nd["sons"][1]]["bb"][:, 0])
            hi = np.maximum(nodes[nd["sons"][0]]["bb"][:, 1], nodes[nd["sons"][1]]["bb"][:, 1])
        else:
            pts = P[:, idx[nd["begin"]:nd["begin"] + nd["size"]]]
            lo, hi = pts.min(1), pts.max(1)
        ext = hi - lo
        flat = (hi - lo) < 2e2 * EPS
        hi = np.where(flat, hi + 1e2 * EPS, hi)
        lo = np.where(flat, lo - 1e2 * EPS, lo)
        ext = np.where(flat, hi - lo, ext)
        nd["bb"] = np.stack([lo, hi, ext], 1)
    # level order ids
    order, h = [0], 0
    while h < len(order):
        order += nodes[order[h]]["sons"]
        h += 1
    bid = {k: i for i, k in enumerate(order)}
    return nodes, idx, order, bid


def norm_seq(v):
    s = v[0] * v[0]
    for t in v[1:]:
        s = s + t * t
    return float(np.sqrt(s))


def pattern(nodes, bid, q, eta):
    far, near = [], []
    stack = [(0, 0)]
    while stack:
        i, j = stack.pop()
        a, b = nodes[i], nodes[j]
        r1 = 0.5 * norm_seq(a["bb"][:, 2])
        r2 = 0.5 * norm_seq(b["bb"][:, 2])
        v = 0.5 * (a["bb"][:, 0] - b["bb"][:, 0] + a["bb"][:, 1] - b["bb"][:, 1])
        dist = norm_seq(v) - r1 - r2
        dist = dist if dist > 0 else 0.0
        radius = r1 if r1 > r2 else r2
        if radius > eta * dist:
            if not a["sons"] or not b["sons"]:
                near.append((bid[i], bid[j]))
            else:
                for jj in b["sons"]:
                    for ii in a["sons"]:
                        stack.append((ii, jj))
        else:
            if (q * q) % 2**32 < (a["size"] * b["size"]) % 2**32:
                far.append((bid[i], bid[j]))
            else:
                near.append((bid[i], bid[j]))
    return far, near


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def fingerprint(name, n, dim, deg, m, eta, kind):
    P = cloud(kind, n, dim)
    q = (deg + 1) ** dim
    nodes, idx, order, bid = build_tree(P, max(m, q))
    far, near = pattern(nodes, bid, q, eta)
    far.sort()
    near.sort()
    meta = np.array([[nodes[k]["begin"], nodes[k]["size"], nodes[k]["level"]] for k in order],
                    dtype=np.int32)
    bbs = np.array([nodes[k]["bb"].T for k in order], dtype=np.float64)  # C x 3 x dim
    near_pairs = int(sum(nodes[order[i]]["size"] * nodes[order[j]]["size"] for i, j in near))
    out = dict(n=n, dim=dim, degree=deg, min_leaf=m, eta=eta, cloud=kind,
               clusters=len(nodes), far_blocks=len(far), near_blocks=len(near),
               near_pairs=near_pairs, perm_sha=sha(idx.astype(np.uint32)),
               meta_sha=sha(meta), bb_sha=sha(bbs),
               far_sha=sha(np.array(far, dtype=np.int32).reshape(-1, 2)),
               near_sha=sha(np.array(near, dtype=np.int32).reshape(-1, 2)))
    if n <= 300:
        out["perm"] = idx.tolist()
    return name, out


def main():
    res = {}
    for case in CASES:
        name, fp = fingerprint(*case)
        res[name] = fp
        print(name, fp["clusters"], fp["far_blocks"], fp["near_blocks"], fp["near_pairs"])
    with open(os.path.join(HERE, "structure.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    main()
