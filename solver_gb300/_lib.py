"""ctypes binding of ``lib/libpeec_gb300.so`` (the C ABI in include/peec_gb300.h).

Loading fails loudly: there is no CPU fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import build as _build

LIB_PATH = _build.LIBDIR / "libpeec_gb300.so"

PEEC_OK = 0
ERRORS = {-1: "PEEC_ERR_CUDA", -2: "PEEC_ERR_OOM", -3: "PEEC_ERR_CANCELLED",
          -4: "PEEC_ERR_TIMEOUT", -5: "PEEC_ERR_BADARG", -6: "PEEC_ERR_UNSUPPORTED",
          -7: "PEEC_ERR_STATE"}

# every symbol declared in include/peec_gb300.h
EXPORTS = ("peec_version", "peec_ctx_create", "peec_ctx_destroy", "peec_last_error",
           "peec_set_topology", "peec_set_incidence", "peec_set_dense", "peec_set_dense_rcc",
           "peec_set_dense_rcc_frequency", "peec_ris_fill", "peec_dense_get",
           "peec_set_edge_state",
           "peec_set_frequency_device", "peec_set_pdiag", "peec_set_rows", "peec_fill",
           "peec_set_frequency", "peec_matvec", "peec_matvec_dev", "peec_port_rhs",
           "peec_gmres", "peec_solve_mixed", "peec_set_stop_flag", "peec_set_device_loop",
           "peec_device_loop_stats", "peec_last_timing",
           "peec_launch_count", "peec_sizes", "peec_stream", "peec_conv_count",
           "peec_conv_info", "peec_zpass_tuning", "peec_set_zpass_forms", "peec_profile_matvec", "peec_multidot",
           "peec_multidot_noalloc", "peec_set_residual_precision",
           "peec_set_lu_component_max", "peec_adjoint", "peec_check_wait_limit",
           "peec_fill_rcc", "peec_set_rows_rcc", "peec_set_rcc_frequency",
           "peec_lu_refactor_setup", "peec_set_frequency_refactor",
           "peec_mesh_gpu_build", "peec_mesh_gpu_len", "peec_mesh_gpu_copy", "peec_mesh_gpu_free")


PREC_FP64, PREC_FP32, PREC_FF = 0, 1, 2


class PeecError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class PeecCancelled(PeecError):
    pass


_lib = None

P = ctypes.c_void_p
I64P = ctypes.POINTER(ctypes.c_int64)
DP = ctypes.POINTER(ctypes.c_double)


def load(build_if_missing: bool = True):
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA extension first")
        _build.build_cuda()
    L = ctypes.CDLL(str(LIB_PATH))
    for name in EXPORTS:
        if not hasattr(L, name):
            raise RuntimeError(f"libpeec_gb300.so does not export {name}")
    L.peec_version.restype = ctypes.c_int
    L.peec_set_residual_precision.argtypes = [P, ctypes.c_int]
    L.peec_set_lu_component_max.argtypes = [P, ctypes.c_int]
    L.peec_check_wait_limit.argtypes = [P]
    L.peec_adjoint.argtypes = [P, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                               ctypes.c_int64, ctypes.c_void_p]
    L.peec_ctx_create.argtypes = [ctypes.POINTER(P), ctypes.c_int]
    L.peec_ctx_destroy.argtypes = [P]
    L.peec_ctx_destroy.restype = None
    L.peec_last_error.argtypes = [P]
    L.peec_last_error.restype = ctypes.c_char_p
    L.peec_set_topology.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                    ctypes.c_int64, ctypes.c_int64, P, P, P, ctypes.c_int64, P, P,
                                    P, ctypes.c_int64]
    L.peec_set_incidence.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, P, P,
                                     ctypes.c_int64, P, ctypes.c_int64]
    L.peec_set_dense.argtypes = [P, P, P, P, P]
    L.peec_set_dense_rcc.argtypes = [P, P, P, P, P]
    L.peec_set_dense_rcc_frequency.argtypes = [P, ctypes.c_double]
    L.peec_ris_fill.argtypes = [P, P, P, P, ctypes.c_double, P, P, P, ctypes.c_double,
                                ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
    L.peec_dense_get.argtypes = [P, ctypes.c_int, ctypes.c_int, P]
    L.peec_set_edge_state.argtypes = [P, P, P, P, P, P, ctypes.c_int64, ctypes.c_double,
                                      ctypes.c_double]
    L.peec_set_frequency_device.argtypes = [P, ctypes.c_double, ctypes.c_int64, P, P, P]
    L.peec_set_pdiag.argtypes = [P, P]
    L.peec_set_rows.argtypes = [P, ctypes.POINTER(P)]
    L.peec_fill.argtypes = [P, P, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                            ctypes.c_double, ctypes.c_double, ctypes.POINTER(P)]
    L.peec_fill_rcc.argtypes = [P, P, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double, ctypes.POINTER(P)]
    L.peec_set_rows_rcc.argtypes = [P, ctypes.POINTER(P), P, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double]
    L.peec_set_rcc_frequency.argtypes = [P, ctypes.c_double]
    L.peec_lu_refactor_setup.argtypes = [P, ctypes.c_int64, P, P]
    L.peec_mesh_gpu_build.restype = ctypes.c_void_p
    L.peec_mesh_gpu_build.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
    L.peec_mesh_gpu_len.restype = ctypes.c_int64
    L.peec_mesh_gpu_len.argtypes = [P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
    L.peec_mesh_gpu_copy.argtypes = [P, ctypes.c_char_p, P]
    L.peec_mesh_gpu_free.argtypes = [P]
    L.peec_mesh_gpu_free.restype = None
    L.peec_set_frequency_refactor.argtypes = [P, ctypes.c_double, P, ctypes.c_int64, P, P, P]
    L.peec_set_frequency.argtypes = [P, ctypes.c_double, P, ctypes.c_int64, P, P, P, P, P, P, P,
                                     P, P, P, P, P]
    L.peec_matvec.argtypes = [P, P, P, ctypes.c_int]
    L.peec_matvec_dev.argtypes = [P, P, P, ctypes.c_int]
    L.peec_port_rhs.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_double, P]
    L.peec_gmres.argtypes = [P, P, P, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                             ctypes.c_int, ctypes.POINTER(ctypes.c_int), DP,
                             ctypes.POINTER(ctypes.c_int), DP, ctypes.c_int,
                             ctypes.POINTER(ctypes.c_int)]
    L.peec_solve_mixed.argtypes = [P, P, P, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_int, ctypes.POINTER(ctypes.c_int), DP,
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.peec_set_stop_flag.argtypes = [P, P]
    L.peec_set_device_loop.argtypes = [P, ctypes.c_int]
    L.peec_device_loop_stats.argtypes = [P, I64P, I64P]
    L.peec_last_timing.argtypes = [P, DP, DP, DP]
    L.peec_launch_count.argtypes = [P]
    L.peec_launch_count.restype = ctypes.c_int64
    L.peec_sizes.argtypes = [P, I64P, I64P, I64P]
    L.peec_stream.argtypes = [P]
    L.peec_stream.restype = ctypes.c_void_p
    L.peec_conv_count.argtypes = [P]
    IP = ctypes.POINTER(ctypes.c_int)
    L.peec_conv_info.argtypes = [P, ctypes.c_int, IP, IP, IP, IP]
    L.peec_zpass_tuning.argtypes = [P, IP, DP, DP]
    L.peec_set_zpass_forms.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.peec_profile_matvec.argtypes = [P, ctypes.c_int, ctypes.c_int, DP]
    L.peec_multidot.argtypes = [P, P, ctypes.c_int64, P, ctypes.c_int64, ctypes.c_int, P]
    L.peec_multidot_noalloc.argtypes = [P, ctypes.c_int64, P, ctypes.c_int64, ctypes.c_int, P, P]
    _lib = L
    return L


def ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def check(ctx, rc):
    if rc != PEEC_OK:
        msg = load().peec_last_error(ctx).decode(errors="replace")
        if rc == -3:
            raise PeecCancelled(rc, msg)
        raise PeecError(rc, msg)
