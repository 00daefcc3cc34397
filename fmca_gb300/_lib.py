"""ctypes binding of the C ABI declared in ``include/fmca_gb300.h``.

The shared library is built in-tree by ``fmca_gb300.build.build()``.  There
is no fallback: if the library is missing or fails to load, importing the
package's compute entry points raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfmca_gb300.so")

FMCA_OK = 0
STATUS_NAMES = {
    0: "FMCA_OK",
    1: "FMCA_ERR_INVALID_ARGUMENT",
    2: "FMCA_ERR_UNSUPPORTED",
    3: "FMCA_ERR_CUDA",
    4: "FMCA_ERR_OUT_OF_MEMORY",
    5: "FMCA_ERR_TIMEOUT",
    6: "FMCA_ERR_INTERNAL",
}

PREC_FP64 = 0
PREC_MIXED = 1
PREC_FP32 = 2
DTYPE_F64 = 0
DTYPE_F32 = 1
ORDER_NATURAL = 0
ORDER_CLUSTER = 1

INFO_KEYS = [
    "n_rows", "n_cols", "dim", "degree", "q", "row_clusters", "col_clusters",
    "far_blocks", "near_blocks", "near_pairs", "row_levels", "col_levels",
    "row_leaves", "col_leaves", "min_leaf", "interpolator",
]
INTERPOLATORS = {"tensor": 0, "total_degree": 1}
INFO_COUNT = 16

# every symbol the header declares; tests check the library exports them all
EXPORTED = [
    "fmca_last_error", "fmca_version", "fmca_kernel_type_from_name",
    "fmca_plan_create", "fmca_plan_destroy", "fmca_plan_info",
    "fmca_plan_statistics", "fmca_plan_permutation", "fmca_plan_clusters",
    "fmca_plan_blocks", "fmca_matvec_workspace_size", "fmca_matvec",
    "fmca_matvec_host", "fmca_plan_check_device_error", "fmca_kernel_eval",
    "fmca_plan_set_profiling", "fmca_plan_profile", "fmca_matvec_static_scratch",
    "fmca_matvec_adjoint_workspace_size", "fmca_matvec_adjoint", "fmca_plan_update_points",
    "fmca_plan_create_batched", "fmca_matvec_graph_create", "fmca_graph_launch",
    "fmca_graph_destroy", "fmca_plan_create_ex", "fmca_plan_interpolator",
    "fmca_plan_save", "fmca_plan_load", "fmca_plan_cloud_offsets", "fmca_plan_device_bytes",
    "fmca_plan_set_wait_limit", "fmca_plan_set_stalled_wait", "fmca_plan_set_autotune",
    "fmca_plan_tuned_config", "fmca_plan_create_gpu", "fmca_plan_set_tuned_config",
    "fmca_plan_assembled_size", "fmca_plan_assemble", "fmca_matvec_assembled",
    "fmca_plan_release_assembled", "fmca_plan_near_packed",
]
TUNE_KEYS = ["tuned", "near_stages", "near_unit", "far_pairs", "far_grid_stages",
             "far_grid_unit", "far_node_stages", "far_node_unit", "wide_below", "slice_below",
             "small_r_tensor", "near_halves", "near_persist", "far_persist", "tune_us",
             "tunings", "far_kron", "near_pack"]
STAGES = ["gather", "leafmom", "m2m", "far", "l2l", "leafgather", "near", "scatter"]


class FmcaError(RuntimeError):
    """A non-OK status returned by the C ABI."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class KernelDesc(C.Structure):
    _fields_ = [("type", C.c_int), ("l", C.c_double), ("c", C.c_double),
                ("nu", C.c_double), ("sigma2", C.c_double)]


_lib = None


def load() -> C.CDLL:
    """Loads the library once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` "
            "(or fmca_gb300.build.build()); there is no CPU fallback")
    lib = C.CDLL(LIB_PATH)
    vp, dp, i64, i32 = C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.c_int
    lib.fmca_last_error.restype = C.c_char_p
    lib.fmca_version.restype = C.c_char_p
    lib.fmca_kernel_type_from_name.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    lib.fmca_plan_create.argtypes = [dp, i32, i64, dp, i64, i32, C.c_double, i64,
                                     C.POINTER(vp)]
    lib.fmca_plan_create_ex.argtypes = [dp, i32, i64, dp, i64, i32, i32, C.c_double, i64,
                                        C.POINTER(vp)]
    lib.fmca_plan_create_gpu.argtypes = [dp, i32, i64, dp, i64, i32, i32, C.c_double, i64,
                                         C.POINTER(C.c_int), C.POINTER(vp)]  # gpu_parts[2]
    lib.fmca_plan_interpolator.argtypes = [vp, dp, dp]
    lib.fmca_plan_save.argtypes = [vp, C.c_char_p]
    lib.fmca_plan_load.argtypes = [C.c_char_p, C.POINTER(vp)]
    lib.fmca_plan_cloud_offsets.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int)]
    lib.fmca_plan_destroy.argtypes = [vp]
    lib.fmca_plan_info.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.fmca_plan_statistics.argtypes = [vp, dp]
    lib.fmca_plan_permutation.argtypes = [vp, i32, C.POINTER(C.c_uint32)]
    lib.fmca_plan_clusters.argtypes = [vp, i32, C.POINTER(C.c_int32), dp]
    lib.fmca_plan_blocks.argtypes = [vp, i32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    lib.fmca_plan_near_packed.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                          C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    lib.fmca_matvec_workspace_size.argtypes = [vp, i32, i32, C.POINTER(C.c_size_t)]
    lib.fmca_matvec.argtypes = [vp, C.POINTER(KernelDesc), i32, i32, i32, i32,
                                vp, i64, i64, vp, i64, i64, vp, C.c_size_t, vp]
    lib.fmca_matvec_host.argtypes = [vp, C.POINTER(KernelDesc), i32, i32, i32, dp, dp]
    lib.fmca_plan_check_device_error.argtypes = [vp]
    lib.fmca_kernel_eval.argtypes = [C.POINTER(KernelDesc), i32, dp, i64, dp, i64, dp]
    lib.fmca_matvec_static_scratch.argtypes = [vp, C.POINTER(KernelDesc), i32, i32, i32,
                                               i32, vp, i64, i64, vp, i64, i64, vp]
    lib.fmca_matvec_adjoint_workspace_size.argtypes = [vp, i32, i32, C.POINTER(C.c_size_t)]
    lib.fmca_matvec_adjoint.argtypes = [vp, C.POINTER(KernelDesc), i32, i32, i32, vp, i64, i64,
                                        vp, i64, i64, vp, vp, i64, i64, vp, vp, vp, C.c_size_t,
                                        vp]
    lib.fmca_plan_update_points.argtypes = [vp, dp, dp]
    lib.fmca_plan_create_batched.argtypes = [C.POINTER(dp), C.POINTER(C.c_int64), i32, i32,
                                             i32, C.c_double, i64, C.POINTER(vp)]
    lib.fmca_matvec_graph_create.argtypes = [vp, C.POINTER(KernelDesc), i32, i32, i32, i32,
                                             vp, i64, i64, vp, i64, i64, vp, C.c_size_t,
                                             C.POINTER(vp)]
    lib.fmca_graph_launch.argtypes = [vp, vp]
    lib.fmca_graph_destroy.argtypes = [vp]
    lib.fmca_plan_set_profiling.argtypes = [vp, i32]
    lib.fmca_plan_profile.argtypes = [vp, dp, C.POINTER(C.c_int64)]
    lib.fmca_plan_device_bytes.argtypes = [vp, C.POINTER(C.c_size_t)]
    lib.fmca_plan_set_wait_limit.argtypes = [vp, C.c_uint64]
    lib.fmca_plan_set_stalled_wait.argtypes = [vp, i32]
    lib.fmca_plan_set_autotune.argtypes = [vp, i32]
    lib.fmca_plan_tuned_config.argtypes = [vp, i32, i32, i32, C.POINTER(C.c_int32)]
    lib.fmca_plan_set_tuned_config.argtypes = [vp, i32, i32, i32, C.POINTER(C.c_int32)]
    lib.fmca_plan_assembled_size.argtypes = [vp, i32, C.POINTER(C.c_size_t)]
    lib.fmca_plan_assemble.argtypes = [vp, C.POINTER(KernelDesc), i32, vp]
    lib.fmca_matvec_assembled.argtypes = [vp, i32, i32, i32, i32, vp, i64, i64, vp, i64, i64,
                                          vp, C.c_size_t, vp]
    lib.fmca_plan_release_assembled.argtypes = [vp]
    for name in EXPORTED:
        if name not in ("fmca_last_error", "fmca_version"):
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != FMCA_OK:
        msg = load().fmca_last_error()
        raise FmcaError(status, msg.decode() if msg else "")
