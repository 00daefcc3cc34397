"""Host-side mirror of FMCA's Python H2 interface on top of the C ABI.

``CovarianceKernel`` and ``H2Matrix`` keep the names, argument meaning and
defaults of the reference's pybind module (py/FMCA.cpp:209-250, 448-468):

    cov = CovarianceKernel("MATERN32", 0.5)
    H = H2Matrix(cov, P, P, 4, 0.8)      # P: dim x n, float64
    y = H.action(x)                      # x: n x R, natural order
    H.statistics()                       # (6, 1): m, n, #LR, #dense, nz/row, GB

Differences, all additive: the interpolation defaults to the Chebyshev
tensor-product interpolator; ``interpolator="total_degree"`` selects the
total-degree one that the reference's pybind module instantiates
(py/FMCA.cpp:37-40); ``min_leaf`` and ``precision`` keyword arguments; ``CovarianceKernel``
accepts a variance ``sigma2``; ``action`` also takes torch tensors (CPU or
CUDA) and returns the same kind of tensor.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import _lib
from ._lib import KernelDesc, check

_PREC = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED, "fp32": _lib.PREC_FP32}


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class CovarianceKernel:
    """Radial covariance kernel, like FMCA's CovarianceKernel(type, l, c, nu)."""

    def __init__(self, ktype: str = "EXPONENTIAL", l: float = 1.0, c: float = 1.0,
                 nu: float = 1.0, sigma2: float = 1.0):
        lib = _lib.load()
        t = C.c_int(0)
        check(lib.fmca_kernel_type_from_name(str(ktype).encode(), C.byref(t)))
        self._type = t.value
        self._name = str(ktype).upper()
        self.l = float(l)
        self.c = float(c)
        self.nu = float(nu)
        self.sigma2 = float(sigma2)

    def kernelType(self) -> str:  # noqa: N802 (reference name)
        return self._name

    @property
    def type_code(self) -> int:
        return self._type

    def desc(self) -> KernelDesc:
        return KernelDesc(self._type, self.l, self.c, self.nu, self.sigma2)

    def eval(self, PR, PC) -> np.ndarray:
        """Dense K(PR, PC): PR dim x n_r, PC dim x n_c; FP64 on the GPU."""
        PR = np.asfortranarray(PR, dtype=np.float64)
        PC = np.asfortranarray(PC, dtype=np.float64)
        if PR.ndim != 2 or PC.ndim != 2 or PR.shape[0] != PC.shape[0]:
            raise ValueError("PR and PC must be dim x n arrays of the same dim")
        out = np.empty((PR.shape[1], PC.shape[1]), dtype=np.float64, order="F")
        d = self.desc()
        check(_lib.load().fmca_kernel_eval(C.byref(d), PR.shape[0], _dptr(PR), PR.shape[1],
                                           _dptr(PC), PC.shape[1], _dptr(out)))
        return out


class H2Matrix:
    """Matrix-free H2 approximation of K(Pr, Pc) with a GPU matvec.

    Mirrors pyH2Matrix(ker, Pr, Pc, p=3, eta=0.8) (py/FMCA.cpp:209-220).
    Keywords: ``min_leaf`` (minimum cluster size; the effective value is
    max(min_leaf, q) like H2ClusterTree::init), ``precision`` ("fp64",
    "fp32" or "mixed"; the default of ``action``), ``interpolator``
    ("tensor": Chebyshev tensor product, q = (p+1)^dim; "total_degree":
    TotalDegreeInterpolator, q = binom(p+dim, dim), as the reference module
    builds it) and ``build`` ("host", or "gpu": the cluster trees' sorts and
    the block pattern on the current CUDA device, fmca_plan_create_gpu, the
    same plan; ``trees_on_gpu`` and ``pattern_on_gpu`` tell what ran
    there). ``fmca_gb300.FMCA`` gives the reference module's defaults.
    """

    def __init__(self, cov: CovarianceKernel, Pr, Pc=None, p: int = 3,
                 eta: float = 0.8, min_leaf: int = 0, precision: str = "mixed",
                 interpolator: str = "tensor", build: str = "host"):
        lib = _lib.load()
        self.cov = cov
        self.p = int(p)
        self.eta = float(eta)
        if interpolator not in _lib.INTERPOLATORS:
            raise ValueError("interpolator must be 'tensor' or 'total_degree'")
        self.interpolator = interpolator
        if precision not in _PREC:
            raise ValueError("precision must be 'fp64', 'fp32' or 'mixed'")
        self.precision = precision
        Pr = np.asfortranarray(Pr, dtype=np.float64)
        if Pr.ndim != 2:
            raise ValueError("Pr must be a dim x n array")
        same = Pc is None or Pc is Pr
        if not same:
            Pc = np.asfortranarray(Pc, dtype=np.float64)
            if Pc.ndim != 2 or Pc.shape[0] != Pr.shape[0]:
                raise ValueError("Pc must be a dim x n array with the dim of Pr")
            same = Pc.shape == Pr.shape and np.array_equal(Pc, Pr)
        self.dim = Pr.shape[0]
        handle = C.c_void_p()
        Pcp = None if same else _dptr(Pc)
        nc = Pr.shape[1] if same else Pc.shape[1]
        if build == "host":
            check(lib.fmca_plan_create_ex(_dptr(Pr), self.dim, Pr.shape[1], Pcp, nc,
                                          _lib.INTERPOLATORS[interpolator], self.p, self.eta,
                                          int(min_leaf), C.byref(handle)))
            self.trees_on_gpu = self.pattern_on_gpu = 0
        elif build == "gpu":
            parts = (C.c_int * 2)()
            check(lib.fmca_plan_create_gpu(_dptr(Pr), self.dim, Pr.shape[1], Pcp, nc,
                                           _lib.INTERPOLATORS[interpolator], self.p, self.eta,
                                           int(min_leaf), parts, C.byref(handle)))
            self.trees_on_gpu, self.pattern_on_gpu = parts[0], parts[1]
        else:
            raise ValueError("build must be 'host' or 'gpu'")
        self._h = handle
        info = (C.c_int64 * _lib.INFO_COUNT)()
        check(lib.fmca_plan_info(self._h, info))
        self.info = {k: int(info[i]) for i, k in enumerate(_lib.INFO_KEYS)}
        self._ws = {}
        # the row points the plan holds (one point cloud), never modified in
        # place: update_points replaces the array
        self._points = np.array(Pr, order="F", copy=True) if same else None

    @classmethod
    def batched(cls, cov: CovarianceKernel, clouds, p: int = 3, eta: float = 0.8,
                min_leaf: int = 0, precision: str = "mixed") -> "H2Matrix":
        """Block-diagonal H2 matrix of independent point clouds (each dim x n_i).

        Right-hand sides are the clouds' vectors stacked in cloud order;
        ``offsets[i]`` is the first row of cloud i.  Every stage of a matvec
        covers all clouds with one kernel launch."""
        lib = _lib.load()
        if precision not in _PREC:
            raise ValueError("precision must be 'fp64', 'fp32' or 'mixed'")
        arrs = [np.asfortranarray(P, dtype=np.float64) for P in clouds]
        if not arrs or any(a.ndim != 2 or a.shape[0] != arrs[0].shape[0] for a in arrs):
            raise ValueError("clouds must be dim x n arrays of one dim")
        self = cls.__new__(cls)
        self.cov, self.p, self.eta, self.precision = cov, int(p), float(eta), precision
        self.interpolator = "tensor"
        self.dim = arrs[0].shape[0]
        ptrs = (C.POINTER(C.c_double) * len(arrs))(*[_dptr(a) for a in arrs])
        ns = (C.c_int64 * len(arrs))(*[a.shape[1] for a in arrs])
        handle = C.c_void_p()
        check(lib.fmca_plan_create_batched(ptrs, ns, len(arrs), self.dim, self.p, self.eta,
                                           int(min_leaf), C.byref(handle)))
        self._h = handle
        info = (C.c_int64 * _lib.INFO_COUNT)()
        check(lib.fmca_plan_info(self._h, info))
        self.info = {k: int(info[i]) for i, k in enumerate(_lib.INFO_KEYS)}
        self._ws = {}
        self.offsets = np.concatenate([[0], np.cumsum([a.shape[1] for a in arrs])])
        return self

    def save(self, path) -> None:
        """Writes the plan to a file (fmca_plan_save): points, trees, block
        lists and interpolation data, not the kernel or the precision."""
        check(_lib.load().fmca_plan_save(self._h, os.fsencode(path)))

    @classmethod
    def load(cls, path, cov: CovarianceKernel, precision: str = "mixed") -> "H2Matrix":
        """A plan written by ``save`` (fmca_plan_load), without rebuilding the
        trees or the block pattern; kernel and precision are chosen anew."""
        lib = _lib.load()
        if precision not in _PREC:
            raise ValueError("precision must be 'fp64', 'fp32' or 'mixed'")
        self = cls.__new__(cls)
        handle = C.c_void_p()
        check(lib.fmca_plan_load(os.fsencode(path), C.byref(handle)))
        self._h = handle
        info = (C.c_int64 * _lib.INFO_COUNT)()
        check(lib.fmca_plan_info(self._h, info))
        self.info = {k: int(info[i]) for i, k in enumerate(_lib.INFO_KEYS)}
        self.cov, self.precision = cov, precision
        self.p, self.dim, self.eta = self.info["degree"], self.info["dim"], None
        self.interpolator = "total_degree" if self.info["interpolator"] == 1 else "tensor"
        self._ws = {}
        self.offsets = self.cloud_offsets()
        return self

    def cloud_offsets(self) -> np.ndarray:
        """First row of every point cloud, then the row count
        (fmca_plan_cloud_offsets); [0, n] for a plan of one cloud."""
        lib = _lib.load()
        cnt = C.c_int(0)
        check(lib.fmca_plan_cloud_offsets(self._h, None, C.byref(cnt)))
        out = np.zeros(cnt.value + 1, dtype=np.int64)
        check(lib.fmca_plan_cloud_offsets(self._h, out.ctypes.data_as(C.POINTER(C.c_int64)),
                                          C.byref(cnt)))
        return out

    def graph(self, x, y, precision: Optional[str] = None) -> "MatvecGraph":
        """Records y = K x for these CUDA tensors into a CUDA graph."""
        return MatvecGraph(self, x, y, precision or self.precision)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().fmca_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def rows(self) -> int:
        return self.info["n_rows"]

    def cols(self) -> int:
        return self.info["n_cols"]

    # -- reference methods -------------------------------------------------
    def interpolation_nodes(self):
        """(nodes dim x q on [0, 1]^dim, invV q x q or None): the plan's
        interpolation nodes and, for total degree, the inverse Vandermonde
        matrix of its Legendre basis at those nodes."""
        q = self.info["q"]
        nodes = np.zeros((self.dim, q), order="F")
        invV = np.zeros((q, q), order="F")
        check(_lib.load().fmca_plan_interpolator(self._h, _dptr(nodes), _dptr(invV)))
        return nodes, (invV if self.interpolator == "total_degree" else None)

    def statistics(self, verbose: bool = True) -> np.ndarray:
        out = np.zeros(6, dtype=np.float64)
        check(_lib.load().fmca_plan_statistics(self._h, _dptr(out)))
        if verbose:
            print(f"matrix size:                  {int(out[0])} x {int(out[1])}")
            print(f"number of low rank blocks:    {int(out[2])}")
            print(f"number of full blocks:        {int(out[3])}")
            print(f"nz per row:                   {out[4]:g}")
            print(f"storage size:                 {out[5]:g}GB")
        return out.reshape(6, 1)

    def _perm(self, side: int) -> np.ndarray:
        n = self.info["n_rows"] if side == 0 else self.info["n_cols"]
        out = np.empty(n, dtype=np.uint32)
        check(_lib.load().fmca_plan_permutation(
            self._h, side, out.ctypes.data_as(C.POINTER(C.c_uint32))))
        return out

    def rindices(self) -> np.ndarray:
        return self._perm(0)

    def cindices(self) -> np.ndarray:
        return self._perm(1)

    def clusters(self, side: int = 0):
        """(meta, bb): meta[c] = (begin, size, level, parent); bb[c] = (min, max, ext)."""
        C_ = self.info["row_clusters"] if side == 0 else self.info["col_clusters"]
        meta = np.empty((C_, 4), dtype=np.int32)
        bb = np.empty((C_, 3, self.dim), dtype=np.float64)
        check(_lib.load().fmca_plan_clusters(self._h, side,
                                             meta.ctypes.data_as(C.POINTER(C.c_int32)),
                                             _dptr(bb)))
        return meta, bb

    def blocks(self, kind: int):
        """(rows, cols) cluster ids of the low-rank (0) or dense (1) blocks."""
        n = self.info["far_blocks"] if kind == 0 else self.info["near_blocks"]
        r = np.empty(n, dtype=np.int32)
        c = np.empty(n, dtype=np.int32)
        check(_lib.load().fmca_plan_blocks(self._h, kind,
                                           r.ctypes.data_as(C.POINTER(C.c_int32)),
                                           c.ctypes.data_as(C.POINTER(C.c_int32))))
        return r, c

    def near_packed(self):
        """(groups, intervals) of the packed near field (fmca_plan_near_packed):
        groups[g] = (first target, targets, first interval, end interval,
        targets of the first leaf), intervals[i] = (first source, end source,
        leaves served: bit 0 the first, bit 1 the second); cluster order.
        Empty arrays where the plan has no packed groups."""
        ng, ni = C.c_int64(0), C.c_int64(0)
        lib = _lib.load()
        check(lib.fmca_plan_near_packed(self._h, C.byref(ng), C.byref(ni), None, None))
        groups = np.zeros((ng.value, 5), dtype=np.uint32)
        ivl = np.zeros((ni.value, 3), dtype=np.uint32)
        if ng.value:
            check(lib.fmca_plan_near_packed(
                self._h, C.byref(ng), C.byref(ni),
                groups.ctypes.data_as(C.POINTER(C.c_uint32)),
                ivl.ctypes.data_as(C.POINTER(C.c_uint32))))
        return groups, ivl

    def action(self, rhs, precision: Optional[str] = None, out=None):
        """y = K_H2 rhs in natural order (pyH2Matrix::action).

        numpy input: FP64 host buffers through fmca_matvec_host.  torch input:
        CUDA tensors stay on the device; CPU tensors are copied to the current
        device and the result copied back, into ``out`` when given (a pinned
        ``out`` and a pinned ``rhs`` make both copies asynchronous DMA)."""
        prec = _PREC[precision or self.precision]
        try:
            import torch
        except ImportError:  # pragma: no cover
            torch = None
        if torch is not None and isinstance(rhs, torch.Tensor):
            if rhs.is_cuda:
                return self.matvec(rhs, out, precision=precision)
            dev = torch.device("cuda", torch.cuda.current_device())
            y = self.matvec(rhs.to(dev, non_blocking=True), precision=precision)
            if out is None:
                return y.to("cpu")
            out.copy_(y, non_blocking=True)
            torch.cuda.current_stream(dev).synchronize()
            return out
        x = np.asfortranarray(rhs, dtype=np.float64)
        vec = x.ndim == 1
        if vec:
            x = x.reshape(-1, 1, order="F")
        if x.ndim != 2 or x.shape[0] != self.cols():
            raise ValueError(f"rhs must have {self.cols()} rows")
        y = np.empty((self.rows(), x.shape[1]), dtype=np.float64, order="F")
        d = self.cov.desc()
        check(_lib.load().fmca_matvec_host(self._h, C.byref(d), prec, _lib.ORDER_NATURAL,
                                           x.shape[1], _dptr(x), _dptr(y)))
        return y[:, 0] if vec else y

    # -- device API --------------------------------------------------------
    def workspace_bytes(self, nrhs: int, precision: Optional[str] = None) -> int:
        n = C.c_size_t(0)
        check(_lib.load().fmca_matvec_workspace_size(
            self._h, _PREC[precision or self.precision], int(nrhs), C.byref(n)))
        return int(n.value)

    def matvec(self, x, y=None, precision: Optional[str] = None, order: str = "natural",
               stream=None, workspace=None):
        """Device matvec on torch CUDA tensors (n_cols x R, any strides).

        Runs asynchronously on ``stream`` (default: torch's current stream).
        """
        import torch
        prec = _PREC[precision or self.precision]
        if x.dim() == 1:
            return self.matvec(x.unsqueeze(1), None if y is None else y.unsqueeze(1),
                               precision, order, stream, workspace).squeeze(1)
        if x.dtype not in (torch.float64, torch.float32):
            raise TypeError("x must be float64 or float32")
        if x.shape[0] != self.cols():
            raise ValueError(f"x must have {self.cols()} rows")
        R = x.shape[1]
        dev = x.device
        if y is None:
            y = torch.empty((self.rows(), R), dtype=x.dtype, device=dev)
        if y.dtype != x.dtype or y.shape != (self.rows(), R) or y.device != dev:
            raise ValueError("y must match x in dtype and device and be n_rows x R")
        dt = _lib.DTYPE_F64 if x.dtype == torch.float64 else _lib.DTYPE_F32
        with torch.cuda.device(dev):
            if stream is None:
                stream = torch.cuda.current_stream(dev)
            if workspace is None:
                key = (prec, R, dev.index)
                need = self.workspace_bytes(R, precision)
                ws = self._ws.get(key)
                if ws is None or ws.numel() < need:
                    ws = torch.empty(need, dtype=torch.uint8, device=dev)
                    self._ws[key] = ws
                workspace = ws
            d = self.cov.desc()
            check(_lib.load().fmca_matvec(
                self._h, C.byref(d), prec, dt,
                _lib.ORDER_NATURAL if order == "natural" else _lib.ORDER_CLUSTER, R,
                C.c_void_p(x.data_ptr()), x.stride(0), x.stride(1),
                C.c_void_p(y.data_ptr()), y.stride(0), y.stride(1),
                C.c_void_p(workspace.data_ptr()), workspace.numel(),
                C.c_void_p(stream.cuda_stream)))
        return y

    def update_points(self, Pr, Pc=None) -> None:
        """Moves the points, keeping the tree, boxes, nodes and block lists."""
        Pr = np.asfortranarray(Pr, dtype=np.float64)
        if Pr.shape != (self.dim, self.rows()):
            raise ValueError("Pr must have the shape of the plan's row points")
        Pcp = None
        if Pc is not None:
            Pc = np.asfortranarray(Pc, dtype=np.float64)
            if Pc.shape != (self.dim, self.cols()):
                raise ValueError("Pc must have the shape of the plan's column points")
            Pcp = _dptr(Pc)
        check(_lib.load().fmca_plan_update_points(self._h, _dptr(Pr), Pcp))
        if Pc is None and getattr(self, "_points", None) is not None:
            self._points = np.array(Pr, order="F", copy=True)

    def current_points(self):
        """The point coordinates (dim x n FP64) a plan of one point cloud
        holds now, as last set by the constructor or update_points; None for
        batched and loaded plans."""
        return getattr(self, "_points", None)

    def adjoint(self, x, y, precision: Optional[str] = None, want_dX: bool = True,
                want_Kx: bool = False, want_Ky: bool = False, stream=None):
        """Gradients of f = sum_r y_r^T K x_r on CUDA tensors.

        Returns a dict with ``values`` (f, df/dl, df/dsigma2 as a float64
        CUDA tensor), and when asked ``dX`` (n x dim, natural order),
        ``Kx`` = K x and ``Ky`` = K y.  The tree and boxes stay fixed."""
        import torch
        prec = _PREC[precision or self.precision]
        if x.dim() == 1:
            x = x.unsqueeze(1)
        if y.dim() == 1:
            y = y.unsqueeze(1)
        if x.dtype != y.dtype or x.device != y.device or x.shape[1] != y.shape[1]:
            raise ValueError("x and y must share dtype, device and number of columns")
        if x.shape[0] != self.cols() or y.shape[0] != self.rows():
            raise ValueError("x must have n_cols rows and y n_rows rows")
        dev = x.device
        R = x.shape[1]
        dt = _lib.DTYPE_F64 if x.dtype == torch.float64 else _lib.DTYPE_F32
        out = {"values": torch.zeros(3, dtype=torch.float64, device=dev)}
        dX = torch.empty((self.rows(), self.dim), dtype=x.dtype, device=dev) if want_dX else None
        Kx = torch.empty_like(y) if want_Kx else None
        Ky = torch.empty_like(x) if want_Ky else None
        with torch.cuda.device(dev):
            if stream is None:
                stream = torch.cuda.current_stream(dev)
            nb = C.c_size_t(0)
            check(_lib.load().fmca_matvec_adjoint_workspace_size(self._h, prec, R, C.byref(nb)))
            key = ("adj", prec, R, dev.index)
            ws = self._ws.get(key)
            if ws is None or ws.numel() < nb.value:
                ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
                self._ws[key] = ws
            d = self.cov.desc()
            ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
            check(_lib.load().fmca_matvec_adjoint(
                self._h, C.byref(d), prec, dt, R,
                ptr(x), x.stride(0), x.stride(1), ptr(y), y.stride(0), y.stride(1),
                ptr(out["values"]), ptr(dX), dX.stride(0) if dX is not None else 0,
                dX.stride(1) if dX is not None else 0, ptr(Kx), ptr(Ky),
                ptr(ws), ws.numel(), C.c_void_p(stream.cuda_stream)))
        if dX is not None:
            out["dX"] = dX
        if Kx is not None:
            out["Kx"] = Kx
        if Ky is not None:
            out["Ky"] = Ky
        return out

    def set_profiling(self, enable: bool = True) -> None:
        """CUDA-event timing of the stages of the following matvecs."""
        check(_lib.load().fmca_plan_set_profiling(self._h, 1 if enable else 0))

    def profile(self):
        """(stage -> ms, kernel launches) of the last matvec (waits for it)."""
        ms = np.zeros(len(_lib.STAGES), dtype=np.float64)
        n = C.c_int64(0)
        check(_lib.load().fmca_plan_profile(self._h, _dptr(ms), C.byref(n)))
        return dict(zip(_lib.STAGES, ms.tolist())), int(n.value)

    def set_wait_limit(self, ns: int = 0) -> None:
        """Limit in ns of the bounded waits inside the kernel sums of the
        following matvecs (fmca_plan_set_wait_limit); 0: the default 2 s."""
        check(_lib.load().fmca_plan_set_wait_limit(self._h, int(ns)))

    def set_autotune(self, enable: bool = True) -> None:
        """Autotuner on or off (fmca_plan_set_autotune): the first
        mixed-precision matvec of each (precision, kernel, nrhs) key measures
        the launch shapes and later calls of that key reuse the fastest."""
        check(_lib.load().fmca_plan_set_autotune(self._h, 1 if enable else 0))

    def tuned_config(self, nrhs: int, precision: Optional[str] = None, cov=None) -> dict:
        """Launch shapes a matvec of this key uses now (fmca_plan_tuned_config)."""
        cov = cov or self.cov
        out = (C.c_int32 * len(_lib.TUNE_KEYS))()
        check(_lib.load().fmca_plan_tuned_config(self._h, _PREC[precision or self.precision],
                                                 cov.desc().type, int(nrhs), out))
        return dict(zip(_lib.TUNE_KEYS, [int(v) for v in out]))

    def set_tuned_config(self, nrhs: int, cfg: dict, precision: Optional[str] = None,
                         cov=None) -> None:
        """Launch shapes for a key as if tuned (fmca_plan_set_tuned_config),
        e.g. a dict returned by ``tuned_config`` in an earlier run; the plan
        must have run a matvec on this device."""
        cov = cov or self.cov
        arr = (C.c_int32 * len(_lib.TUNE_KEYS))(*[int(cfg.get(k, 0)) for k in _lib.TUNE_KEYS])
        check(_lib.load().fmca_plan_set_tuned_config(self._h, _PREC[precision or self.precision],
                                                     cov.desc().type, int(nrhs), arr))

    def set_stalled_wait(self, on: bool) -> None:
        """Test hook (fmca_plan_set_stalled_wait): while on, the first wait of
        every kernel-sum CTA runs out after the wait limit."""
        check(_lib.load().fmca_plan_set_stalled_wait(self._h, 1 if on else 0))

    def device_bytes(self) -> int:
        """Device memory the plan holds now (fmca_plan_device_bytes)."""
        n = C.c_size_t(0)
        check(_lib.load().fmca_plan_device_bytes(self._h, C.byref(n)))
        return int(n.value)

    def check_device_error(self) -> None:
        check(_lib.load().fmca_plan_check_device_error(self._h))

    # -- assembled H2 matrix (stored blocks) -------------------------------
    def assembled_bytes(self, precision: Optional[str] = None) -> int:
        """Device bytes the stored blocks of ``computeH2Matrix`` take
        (fmca_plan_assembled_size; FP64 values for "fp64", FP32 otherwise)."""
        n = C.c_size_t(0)
        check(_lib.load().fmca_plan_assembled_size(self._h, _PREC[precision or self.precision],
                                                   C.byref(n)))
        return int(n.value)

    def computeH2Matrix(self, precision: Optional[str] = None, cov=None,  # noqa: N802
                        stream=None) -> None:
        """Evaluates and stores every far-field coupling block and dense
        near-field block on the current CUDA device (H2MatrixBase::
        computeH2Matrix, H2MatrixBase.h:222-255) for the kernel ``cov``
        (default: the matrix's kernel); later products ``H * x`` stream the
        stored blocks instead of evaluating the kernel.  Needs
        ``assembled_bytes(precision)`` of free device memory."""
        import torch
        prec = precision or self.precision
        cov = cov or self.cov
        d = cov.desc()
        if stream is None:
            stream = torch.cuda.current_stream()
        check(_lib.load().fmca_plan_assemble(self._h, C.byref(d), _PREC[prec],
                                             C.c_void_p(stream.cuda_stream)))
        self._asm_prec = prec

    def release_assembled(self) -> None:
        """Frees the stored blocks (fmca_plan_release_assembled)."""
        check(_lib.load().fmca_plan_release_assembled(self._h))
        self._asm_prec = None

    @property
    def assembled(self) -> Optional[str]:
        """Precision the stored blocks serve ("fp64", or "fp32" / "mixed"),
        None without stored blocks."""
        return getattr(self, "_asm_prec", None)

    def mul(self, x, y=None, precision: Optional[str] = None, order: str = "natural",
            stream=None, workspace=None):
        """Device product with the stored blocks (fmca_matvec_assembled) on
        torch CUDA tensors, arguments as for ``matvec``; the precision
        defaults to the one the blocks were assembled in."""
        import torch
        prec_name = precision or self.assembled or self.precision
        prec = _PREC[prec_name]
        if x.dim() == 1:
            return self.mul(x.unsqueeze(1), None if y is None else y.unsqueeze(1),
                            precision, order, stream, workspace).squeeze(1)
        if x.dtype not in (torch.float64, torch.float32):
            raise TypeError("x must be float64 or float32")
        if x.shape[0] != self.cols():
            raise ValueError(f"x must have {self.cols()} rows")
        R = x.shape[1]
        dev = x.device
        if y is None:
            y = torch.empty((self.rows(), R), dtype=x.dtype, device=dev)
        if y.dtype != x.dtype or y.shape != (self.rows(), R) or y.device != dev:
            raise ValueError("y must match x in dtype and device and be n_rows x R")
        dt = _lib.DTYPE_F64 if x.dtype == torch.float64 else _lib.DTYPE_F32
        with torch.cuda.device(dev):
            if stream is None:
                stream = torch.cuda.current_stream(dev)
            if workspace is None:
                key = (prec, R, dev.index)
                need = self.workspace_bytes(R, prec_name)
                ws = self._ws.get(key)
                if ws is None or ws.numel() < need:
                    ws = torch.empty(need, dtype=torch.uint8, device=dev)
                    self._ws[key] = ws
                workspace = ws
            check(_lib.load().fmca_matvec_assembled(
                self._h, prec, dt,
                _lib.ORDER_NATURAL if order == "natural" else _lib.ORDER_CLUSTER, R,
                C.c_void_p(x.data_ptr()), x.stride(0), x.stride(1),
                C.c_void_p(y.data_ptr()), y.stride(0), y.stride(1),
                C.c_void_p(workspace.data_ptr()), workspace.numel(),
                C.c_void_p(stream.cuda_stream)))
        return y

    def __mul__(self, rhs):
        """H * rhs with the stored blocks (H2MatrixBase::operator*,
        H2MatrixBase.h:107-109): natural order; CUDA tensors stay on the
        device, numpy arrays and CPU tensors are copied in and out (FP64)."""
        import torch
        if self.assembled is None:
            raise _lib.FmcaError(1, "the matrix holds no assembled blocks: call "
                                    "computeH2Matrix() first")
        if isinstance(rhs, torch.Tensor) and rhs.is_cuda:
            return self.mul(rhs)
        host = torch.as_tensor(np.asarray(rhs, dtype=np.float64))
        vec = host.dim() == 1
        x = host.reshape(-1, 1) if vec else host
        dev = torch.device("cuda", torch.cuda.current_device())
        y = self.mul(x.to(dev))
        y = y.cpu().numpy()
        if isinstance(rhs, torch.Tensor):
            y = torch.from_numpy(y)
        return y[:, 0] if vec else y

    def full(self, precision: Optional[str] = None, block: int = 64) -> np.ndarray:
        """The H2 matrix as a dense FP64 array (n_rows x n_cols, natural
        order): H * I, in blocks of ``block`` identity columns, like
        H2MatrixBase::full (H2MatrixBase.h:155-158).  Uses the stored blocks
        when the matrix is assembled, else the matrix-free product."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        nc = self.cols()
        out = np.empty((self.rows(), nc), dtype=np.float64, order="F")
        for c0 in range(0, nc, block):
            c1 = min(nc, c0 + block)
            e = torch.zeros((nc, c1 - c0), dtype=torch.float64, device=dev)
            e[torch.arange(c0, c1, device=dev), torch.arange(c1 - c0, device=dev)] = 1.0
            y = self.mul(e, precision=precision) if self.assembled else \
                self.matvec(e, precision=precision)
            out[:, c0:c1] = y.cpu().numpy()
        return out


class MultipoleFunctionEvaluator:
    """Evaluation of a kernel expansion f(y) = sum_j k(y, p_j) c_j at many
    points through an H2 matrix: FMCA's MultipoleFunctionEvaluator
    (FMCA/src/KernelInterpolation/MultipoleFunctionEvaluator.h:17-62), with
    its interpolator (total degree), its defaults (eta = 0, degree 3, minimum
    cluster size 0) and the evaluation points as rows, the data points as
    columns.  ``precision`` chooses the GPU product (FP64 by default, as the
    reference computes)."""

    def __init__(self, kernel: Optional[CovarianceKernel] = None, P=None, Peval=None,
                 eta: float = 0.0, mpole_deg: int = 3, precision: str = "fp64"):
        self.H = None
        if kernel is not None:
            self.init(kernel, P, Peval, eta, mpole_deg, precision)

    def init(self, kernel: CovarianceKernel, P, Peval, eta: float = 0.0, mpole_deg: int = 3,
             precision: str = "fp64") -> None:
        """Trees of both point sets and the block pattern (init, :24-38)."""
        self.eta = float(eta) if eta >= 0 else 0.0
        self.mpole_deg = int(mpole_deg)
        self._P = np.array(P, dtype=np.float64, order="F", copy=True)
        self._Peval = np.array(Peval, dtype=np.float64, order="F", copy=True)
        self.H = H2Matrix(kernel, self._Peval, self._P, self.mpole_deg, self.eta, min_leaf=0,
                          precision=precision, interpolator="total_degree")

    def evaluate(self, P, Peval, C) -> np.ndarray:
        """f at Peval for the coefficients C (n_P x R, natural order), as
        evaluate (:52-58).  Points other than those of ``init`` are moved
        into the trees, boxes and nodes built at ``init``."""
        if self.H is None:
            raise RuntimeError("MultipoleFunctionEvaluator: call init() first")
        P = np.asarray(P, dtype=np.float64)
        Peval = np.asarray(Peval, dtype=np.float64)
        if not (np.array_equal(P, self._P) and np.array_equal(Peval, self._Peval)):
            self.H.update_points(Peval, P)
            self._P = np.array(P, order="F", copy=True)
            self._Peval = np.array(Peval, order="F", copy=True)
        return self.H.action(C)

    def statistics(self, verbose: bool = True) -> np.ndarray:
        return self.H.statistics(verbose)


class MatvecGraph:
    """A matvec recorded into a CUDA graph (fmca_matvec_graph_create); each
    ``launch`` replays the whole product with a single graph launch."""

    def __init__(self, H: H2Matrix, x, y, precision: str):
        import torch
        if not (x.is_cuda and y.is_cuda) or x.dtype != y.dtype:
            raise ValueError("x and y must be CUDA tensors of one dtype")
        self.H, self.x, self.y = H, x, y  # keep the bound buffers alive
        dt = _lib.DTYPE_F64 if x.dtype == torch.float64 else _lib.DTYPE_F32
        self.ws = torch.empty(H.workspace_bytes(x.shape[1], precision), dtype=torch.uint8,
                              device=x.device)
        g = C.c_void_p()
        d = H.cov.desc()
        with torch.cuda.device(x.device):
            check(_lib.load().fmca_matvec_graph_create(
                H.handle, C.byref(d), _PREC[precision], dt, _lib.ORDER_NATURAL, x.shape[1],
                C.c_void_p(x.data_ptr()), x.stride(0), x.stride(1),
                C.c_void_p(y.data_ptr()), y.stride(0), y.stride(1),
                C.c_void_p(self.ws.data_ptr()), self.ws.numel(), C.byref(g)))
        self._g = g

    def launch(self, stream=None):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(self.x.device)
        check(_lib.load().fmca_graph_launch(self._g, C.c_void_p(stream.cuda_stream)))
        return self.y

    def __del__(self):
        g = getattr(self, "_g", None)
        if g:
            try:
                _lib.load().fmca_graph_destroy(g)
            except Exception:
                pass
            self._g = None
