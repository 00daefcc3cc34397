"""ORACLE — test infrastructure only (see h2_oracle.cpp for what it restates
and what pins it).  Loaded by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline legs; never by the fmca_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    lib = C.CDLL(path)
    dp, vp, i64, i32 = C.POINTER(C.c_double), C.c_void_p, C.c_int64, C.c_int
    lib.oracle_plan_create.restype = vp
    lib.oracle_plan_create.argtypes = [dp, i32, i64, dp, i64, i32, C.c_double, i64]
    lib.oracle_plan_create_ex.restype = vp
    lib.oracle_plan_create_ex.argtypes = [dp, i32, i64, dp, i64, i32, C.c_double, i64, i32]
    lib.oracle_interp.restype = i32
    lib.oracle_interp.argtypes = [vp, dp, dp]
    lib.oracle_plan_destroy.argtypes = [vp]
    lib.oracle_counts.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.oracle_perm.argtypes = [vp, i32, C.POINTER(C.c_uint32)]
    lib.oracle_clusters.argtypes = [vp, i32, C.POINTER(C.c_int32), dp]
    lib.oracle_blocks.argtypes = [vp, i32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    lib.oracle_statistics.argtypes = [vp, dp]
    lib.oracle_check_transfer.restype = C.c_double
    lib.oracle_check_transfer.argtypes = [vp]
    lib.oracle_action.argtypes = [vp, i32, C.c_double, C.c_double, C.c_double, dp, i32, dp,
                                  i32, i32, dp]
    lib.oracle_dense_matvec.argtypes = [i32, C.c_double, C.c_double, C.c_double, i32, dp, i64,
                                        dp, i64, dp, i32, dp, i32]
    lib.oracle_adjoint.argtypes = [vp, i32, C.c_double, C.c_double, dp, dp, i32, dp, dp, i32]
    lib.oracle_update_points.argtypes = [vp, dp]
    lib.oracle_set_keep.argtypes = [vp, i32]
    lib.oracle_action_part.argtypes = [vp, i32, C.c_double, C.c_double, C.c_double, dp, i32,
                                       dp, i32, i32, i32, dp, C.POINTER(C.c_int64)]
    lib.oracle_kernel.restype = C.c_double
    lib.oracle_kernel.argtypes = [i32, C.c_double, C.c_double, C.c_double]
    _lib = lib
    return lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OraclePlan:
    """FP64 CPU H2 restatement over the same inputs as fmca_gb300.H2Matrix."""

    def __init__(self, Pr, Pc=None, p=3, eta=0.8, min_leaf=0, interpolator="tensor"):
        lib = load()
        if interpolator not in ("tensor", "total_degree"):
            raise ValueError("interpolator must be 'tensor' or 'total_degree'")
        self.interpolator = interpolator
        self.Pr = np.asfortranarray(Pr, dtype=np.float64)
        self.same = Pc is None
        self.Pc = self.Pr if self.same else np.asfortranarray(Pc, dtype=np.float64)
        self.dim = self.Pr.shape[0]
        self._h = lib.oracle_plan_create_ex(_d(self.Pr), self.dim, self.Pr.shape[1],
                                            None if self.same else _d(self.Pc),
                                            self.Pc.shape[1], int(p), float(eta),
                                            int(min_leaf), int(interpolator == "total_degree"))
        cnt = (C.c_int64 * 6)()
        lib.oracle_counts(self._h, cnt)
        (self.row_clusters, self.col_clusters, self.n_far, self.n_near, self.q,
         self.near_pairs) = list(cnt)

    def interp(self):
        """(nodes dim x q, invV q x q or None for the tensor product)"""
        lib = load()
        nodes = np.zeros((self.dim, self.q), order="F")
        invV = np.zeros((self.q, self.q), order="F")
        lib.oracle_interp(self._h, _d(nodes), _d(invV))
        return nodes, (invV if self.interpolator == "total_degree" else None)

    def __del__(self):
        if getattr(self, "_h", None):
            load().oracle_plan_destroy(self._h)
            self._h = None

    def perm(self, side):
        n = self.Pr.shape[1] if side == 0 else self.Pc.shape[1]
        out = np.empty(n, dtype=np.uint32)
        load().oracle_perm(self._h, side, out.ctypes.data_as(C.POINTER(C.c_uint32)))
        return out

    def clusters(self, side):
        Cn = self.row_clusters if side == 0 else self.col_clusters
        meta = np.empty((Cn, 4), dtype=np.int32)
        bb = np.empty((Cn, 3, self.dim), dtype=np.float64)
        load().oracle_clusters(self._h, side, meta.ctypes.data_as(C.POINTER(C.c_int32)), _d(bb))
        return meta, bb

    def blocks(self, kind):
        n = self.n_far if kind == 0 else self.n_near
        r = np.empty(n, dtype=np.int32)
        c = np.empty(n, dtype=np.int32)
        load().oracle_blocks(self._h, kind, r.ctypes.data_as(C.POINTER(C.c_int32)),
                             c.ctypes.data_as(C.POINTER(C.c_int32)))
        return r, c

    def statistics(self):
        out = np.zeros(6)
        load().oracle_statistics(self._h, _d(out))
        return out

    def update_points(self, P):
        """Moves the points of a one-cloud plan, keeping its structure."""
        assert self.same
        P = np.asfortranarray(P, dtype=np.float64)
        assert P.shape == self.Pr.shape
        load().oracle_update_points(self._h, _d(P))

    def check_transfer(self):
        return load().oracle_check_transfer(self._h)

    def set_keep(self, on=True):
        """Keep x (cluster order) and the moments of the following ``action``
        calls, for ``action_part``."""
        load().oracle_set_keep(self._h, int(bool(on)))

    def action_part(self, ktype, l, x, y, part, nparts, c=1.0, sigma2=1.0, nthreads=0):
        """Rows of one part of the product (oracle_action_part): writes them
        into y (n_r x R, natural order, F-order float64) and returns
        ((first row, row count) in cluster order, (dense_pairs, lr_pairs))."""
        x = np.asfortranarray(x, dtype=np.float64)
        assert y.flags.f_contiguous and y.dtype == np.float64 and y.shape[1] == x.shape[1]
        work = np.zeros(2)
        rows = (C.c_int64 * 2)()
        load().oracle_action_part(self._h, int(ktype), float(l), float(c), float(sigma2), _d(x),
                                  x.shape[1], _d(y), int(part), int(nparts), int(nthreads),
                                  _d(work), rows)
        if rows[0] < 0:
            raise ValueError("action_part: no kept state for this R, or no level with "
                             f"{nparts} clusters")
        return (int(rows[0]), int(rows[1])), tuple(work)

    def action(self, ktype, l, x, c=1.0, sigma2=1.0, bucket_stride=1, nthreads=0):
        """y = sigma2 * H2(x) in natural order; returns (y, (dense_pairs, lr_pairs))."""
        x = np.asfortranarray(x, dtype=np.float64)
        vec = x.ndim == 1
        if vec:
            x = x.reshape(-1, 1, order="F")
        y = np.empty((self.Pr.shape[1], x.shape[1]), dtype=np.float64, order="F")
        work = np.zeros(2)
        load().oracle_action(self._h, int(ktype), float(l), float(c), float(sigma2), _d(x),
                             x.shape[1], _d(y), int(bucket_stride), int(nthreads), _d(work))
        return (y[:, 0] if vec else y), tuple(work)


def adjoint(O: "OraclePlan", ktype, l, x, y, sigma2=1.0, nthreads=0):
    """(f, df/dl, df/dsigma2), dX (n x dim) of f = sum_r y_r^T K x_r for the
    oracle's one-cloud plan, tree and boxes fixed."""
    x = np.asfortranarray(x, dtype=np.float64)
    y = np.asfortranarray(y, dtype=np.float64)
    if x.ndim == 1:
        x = x.reshape(-1, 1, order="F")
        y = y.reshape(-1, 1, order="F")
    vals = np.zeros(3)
    dX = np.zeros((O.Pr.shape[1], O.dim))
    load().oracle_adjoint(O._h, int(ktype), float(l), float(sigma2), _d(x), _d(y), x.shape[1],
                          _d(vals), _d(dX), int(nthreads))
    return vals, dX


def dense_matvec(ktype, l, Pr, Pc, x, c=1.0, sigma2=1.0, nthreads=0):
    Pr = np.asfortranarray(Pr, dtype=np.float64)
    Pc = np.asfortranarray(Pc, dtype=np.float64)
    x = np.asfortranarray(x, dtype=np.float64)
    vec = x.ndim == 1
    if vec:
        x = x.reshape(-1, 1, order="F")
    y = np.empty((Pr.shape[1], x.shape[1]), dtype=np.float64, order="F")
    load().oracle_dense_matvec(int(ktype), float(l), float(c), float(sigma2), Pr.shape[0], _d(Pr),
                               Pr.shape[1], _d(Pc), Pc.shape[1], _d(x), x.shape[1], _d(y),
                               int(nthreads))
    return y[:, 0] if vec else y


def kernel(ktype, l, r, c=1.0):
    return load().oracle_kernel(int(ktype), float(l), float(c), float(r))
