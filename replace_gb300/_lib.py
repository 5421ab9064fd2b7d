"""Loads libgpl_gb300.so (the C ABI of include/gpl.h) with ctypes.

There is no CPU fallback: if the library or a CUDA device is missing, calls
fail with an error instead of computing anything on the host.
"""

from __future__ import annotations

import ctypes as C
import os

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgpl_gb300.so")

_lib = None


class GplError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"gpl status {status}: {message}")
        self.status = status
        self.message = message


def load(build_if_missing: bool = True):
    """Return the loaded library (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise GplError(_abi.GPL_ERR_NO_DEVICE, f"{LIB_PATH} is not built")
        from . import build
        build.build()
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.gpl_version.restype = C.c_char_p
    L.gpl_last_error.restype = C.c_char_p
    L.gpl_params_default.argtypes = [C.POINTER(_abi.Params)]
    L.gpl_create.argtypes = [C.POINTER(_abi.NetlistDesc), C.POINTER(_abi.Params), C.POINTER(vp)]
    L.gpl_destroy.argtypes = [vp]
    L.gpl_initial_place.argtypes = [vp, C.POINTER(_abi.IpStats)]
    L.gpl_nesterov_init.argtypes = [vp, C.POINTER(_abi.JobInfo)]
    L.gpl_set_net_weights.argtypes = [vp, vp, C.c_int64]
    L.gpl_nesterov_run.argtypes = [vp, C.c_int32, C.POINTER(_abi.NesterovStats), C.POINTER(_abi.IterLog)]
    L.gpl_batch_nesterov_run.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32,
                                         C.POINTER(_abi.NesterovStats), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int64)]
    L.gpl_batch_initial_place.argtypes = [C.POINTER(vp), C.c_int32, C.POINTER(_abi.IpStats),
                                          C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    L.gpl_get_inst_locations.argtypes = [vp, vp, vp]
    L.gpl_get_gcell_coords.argtypes = [vp, vp]
    L.gpl_eval.argtypes = [vp, vp, C.c_float, C.c_float, vp, vp, C.POINTER(_abi.EvalStats)]
    L.gpl_get_bins.argtypes = [vp] * 8
    L.gpl_get_gcells.argtypes = [vp] * 4
    L.gpl_poisson_solve.argtypes = [C.c_int32] * 4 + [vp] * 5
    L.gpl_kernel_times.restype = C.c_int32
    L.gpl_kernel_times.argtypes = [vp, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                   C.POINTER(C.c_int64), C.c_int32]
    L.gpl_kernel_times_reset.argtypes = [vp, C.c_int32]
    L.gpl_kernel_launch_count.restype = C.c_int64
    L.gpl_kernel_launch_count.argtypes = [vp]
    L.gpl_server_params_default.argtypes = [C.POINTER(_abi.ServerParams)]
    L.gpl_server_create.argtypes = [C.POINTER(_abi.ServerParams), C.POINTER(vp)]
    L.gpl_server_submit_weighted.argtypes = [vp, C.POINTER(_abi.NetlistDesc), C.POINTER(_abi.Params),
                                             vp, C.c_int64, C.POINTER(C.c_int64)]
    L.gpl_server_submit.argtypes = [vp, C.POINTER(_abi.NetlistDesc), C.POINTER(_abi.Params),
                                    C.POINTER(C.c_int64)]
    L.gpl_server_poll.restype = C.c_int32
    L.gpl_server_poll.argtypes = [vp, C.POINTER(_abi.ServerResult), C.c_int32, C.c_int32]
    L.gpl_server_get_inst_locations.argtypes = [vp, C.c_int64, vp, vp]
    L.gpl_server_release.argtypes = [vp, C.c_int64]
    L.gpl_server_cancel.argtypes = [vp, C.c_int64]
    L.gpl_server_counts.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32)]
    L.gpl_server_destroy.argtypes = [vp]
    for name in ("gpl_server_create", "gpl_server_submit", "gpl_server_submit_weighted",
                 "gpl_server_get_inst_locations",
                 "gpl_server_release", "gpl_server_cancel"):
        getattr(L, name).restype = C.c_int
    for name in ("gpl_create", "gpl_initial_place", "gpl_nesterov_init", "gpl_nesterov_run",
                 "gpl_batch_nesterov_run", "gpl_batch_initial_place",
                 "gpl_set_net_weights",
                 "gpl_get_inst_locations", "gpl_get_gcell_coords", "gpl_eval", "gpl_get_bins",
                 "gpl_get_gcells", "gpl_poisson_solve"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def last_error() -> str:
    return (load().gpl_last_error() or b"").decode()


def check(status: int, allow=()):
    if status != 0 and status not in allow:
        raise GplError(status, last_error())
    return status
