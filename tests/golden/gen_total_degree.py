"""Generates tests/golden/total_degree.json: the interpolation nodes of FMCA's
TotalDegreeInterpolator (DeMarchi points) and the inverse Vandermonde matrix,
from a numpy/scipy restatement independent of the C++ plan builder and of
the C++ oracle.

Followed: FMCA/src/Interpolator/TotalDegreeInterpolator.h:26-47,
FMCA/src/Interpolator/DeMarchiPoints.h:20-43,
FMCA/src/Interpolator/evalPolynomials.h:19-63,
FMCA/src/util/MultiIndexSet.h:39-100 (total-degree criterion, FMCA_Compare
order), FMCA/src/util/HaltonSet.h:30-146 (HaltonSet<100>: 100 points
skipped).

Independent parts: the candidates come from scipy's unscrambled Halton
generator (scipy.stats.qmc.Halton, fast-forwarded by 100 points), the pivot
order from LAPACK's column-pivoted Householder QR (xGEQP3 through
scipy.linalg.qr(pivoting=True), the algorithm family of Eigen's
ColPivHouseholderQR that the reference calls) and invV from numpy's
inverse.

Run:  python tests/golden/gen_total_degree.py
"""
from __future__ import annotations

import itertools
import json
import os

import numpy as np
import scipy.linalg
from scipy.stats import qmc

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [(1, 3), (2, 4), (2, 7), (3, 2), (3, 4), (3, 6)]


def index_set(dim, deg):
    s = [k for k in itertools.product(range(deg + 1), repeat=dim) if sum(k) <= deg]
    return sorted(s, key=lambda k: (sum(k), k))


def legendre(deg, x):
    """L2-normalised Legendre polynomials on [0, 1]: rows 0..deg."""
    out = np.empty((deg + 1,) + np.shape(x))
    p0, p1 = np.zeros_like(x), np.ones_like(x)
    out[0] = 1.0
    for i in range(1, deg + 1):
        v = (2 * i - 1) / i * (2 * x - 1) * p1 - (i - 1) / i * p0
        p0, p1 = p1, v
        out[i] = v * np.sqrt(2 * i + 1)
    return out


def polys(idx, deg, X):
    """q x m matrix of the polynomials at the columns of X (dim x m)."""
    f = [legendre(deg, X[d]) for d in range(X.shape[0])]
    V = np.ones((len(idx), X.shape[1]))
    for k, m in enumerate(idx):
        for d, md in enumerate(m):
            V[k] *= f[d][md]
    return V


def nodes(dim, deg):
    idx = index_set(dim, deg)
    q = len(idx)
    h = qmc.Halton(dim, scramble=False)
    h.fast_forward(100)
    cand = h.random(10 * q).T  # dim x 10 q
    VT = polys(idx, deg, cand)
    _, piv = scipy.linalg.qr(VT, mode="r", pivoting=True)
    Xi = cand[:, piv[:q]]
    V = polys(idx, deg, Xi).T  # V(i, k) = polynomial k at node i
    return Xi, np.linalg.inv(V)


def main():
    out = {}
    for dim, deg in CASES:
        Xi, invV = nodes(dim, deg)
        rec = {"dim": dim, "degree": deg, "q": Xi.shape[1], "nodes": Xi.T.tolist()}
        if Xi.shape[1] <= 35:  # the larger inverses follow from the nodes
            rec["invV"] = invV.tolist()
        out[f"{dim}_{deg}"] = rec
    with open(os.path.join(HERE, "total_degree.json"), "w") as f:
        json.dump(out, f)


if __name__ == "__main__":
    main()
