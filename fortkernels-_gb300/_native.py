"""ctypes binding of libfk_gb300.so (the C ABI of include/fk_abi.h).

The library is the only compute path: if it cannot be loaded, every call
raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfk_gb300.so")

FK_OK, FK_EINVAL, FK_ENOMEM, FK_ECUDA, FK_ETIMEOUT, FK_EBUSY, FK_ENOTSUP, FK_ECANCELED = range(8)
FK_FP64, FK_MIXED = 0, 1
FK_GPP_ROOT_QUIRKS = 0x1
FK_GPP_ACHSTEMP = 0x2
FK_GPP_HALF_SUM = 0x4
FK_GPP_PHYSICS = 0x8
FK_GPP_REAL_ZERO_MASKED = 0x10
FK_FF_SCHDT_GEMM = 0x1
FK_FF_PHYSICS = 0x2
FK_FF_SPLIT_ACHD = 0x4

# Every symbol include/fk_abi.h declares.
SYMBOLS = ("fk_create", "fk_destroy", "fk_set_stream", "fk_synchronize", "fk_reserve", "fk_strerror",
           "fk_last_error", "fk_version", "fk_gpp", "fk_ff", "fk_set_profiling", "fk_last_timings",
           "fk_last_launches", "fk_last_kernel_time", "fk_last_transfer", "fk_gpp_static", "fk_gpp_real", "fk_server_create", "fk_server_destroy",
           "fk_server_resident_put", "fk_server_resident_evict", "fk_server_submit", "fk_server_wait",
           "fk_server_stats", "fk_server_tune", "fk_set_wait_limit", "fk_selftest_timeout", "fk_wait_error_status", "fk_server_cancel",
           "fk_set_error_estimate", "fk_gpp_error_estimate")


class ServerConfig(ctypes.Structure):
    """fk_server_config of include/fk_abi.h."""
    _fields_ = [("hbm_bytes", ctypes.c_size_t), ("max_active", ctypes.c_int), ("step_stages", ctypes.c_int)]


class GppRequest(ctypes.Structure):
    """fk_gpp_request of include/fk_abi.h."""
    _fields_ = [("number_bands", ctypes.c_int), ("nvband", ctypes.c_int), ("ncouls", ctypes.c_int),
                ("ngpown", ctypes.c_int), ("aqsmtemp", ctypes.c_void_p), ("aqsntemp", ctypes.c_void_p),
                ("I_eps_array", ctypes.c_void_p), ("wtilde_array", ctypes.c_void_p),
                ("eps_key", ctypes.c_ulonglong), ("wtilde_key", ctypes.c_ulonglong), ("vcoul", ctypes.c_void_p),
                ("inv_igp_index", ctypes.c_void_p), ("indinv", ctypes.c_void_p), ("wx_array", ctypes.c_void_p),
                ("flags", ctypes.c_uint), ("achtemp", ctypes.c_void_p), ("asxtemp", ctypes.c_void_p),
                ("acht_n1_loc", ctypes.c_void_p)]


class ServerInfo(ctypes.Structure):
    """fk_server_info of include/fk_abi.h."""
    _fields_ = [("submitted", ctypes.c_ulonglong), ("completed", ctypes.c_ulonglong), ("steps", ctypes.c_ulonglong),
                ("p50_s", ctypes.c_double), ("p99_s", ctypes.c_double), ("mean_s", ctypes.c_double),
                ("terms_per_s", ctypes.c_double), ("mean_active", ctypes.c_double), ("peak_active", ctypes.c_int),
                ("hbm_peak_bytes", ctypes.c_size_t)]


class FKError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Load libfk_gb300.so; raise if it is missing (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FKError(FK_ECUDA, f"{path} is missing: build it with __graft_entry__.build() "
                                "(the CUDA library is the only compute path)")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    I, D, U = ctypes.c_int, ctypes.c_double, ctypes.c_uint
    L.fk_create.argtypes = [I, ctypes.POINTER(P)]
    L.fk_destroy.argtypes = [P]
    L.fk_set_stream.argtypes = [P, P]
    L.fk_synchronize.argtypes = [P]
    L.fk_reserve.argtypes = [P, ctypes.c_size_t]
    L.fk_strerror.argtypes = [I]
    L.fk_strerror.restype = ctypes.c_char_p
    L.fk_last_error.argtypes = [P]
    L.fk_last_error.restype = ctypes.c_char_p
    L.fk_version.argtypes = []
    L.fk_version.restype = ctypes.c_char_p
    L.fk_gpp.argtypes = [P, I, I, I, I] + [P] * 8 + [I, U] + [P] * 4
    L.fk_ff.argtypes = [P] + [I] * 6 + [P] * 11 + [D] * 4 + [I, U] + [P] * 6
    L.fk_gpp_static.argtypes = [P, I, I, I, I] + [P] * 8 + [U] + [P] * 4
    L.fk_gpp_real.restype = I
    L.fk_gpp_real.argtypes = [P, I, I, I, I] + [P] * 8 + [I, U] + [P] * 3
    UL = ctypes.c_ulonglong
    L.fk_server_create.argtypes = [I, ctypes.POINTER(ServerConfig), ctypes.POINTER(P)]
    L.fk_server_destroy.argtypes = [P]
    L.fk_server_resident_put.argtypes = [P, UL, P, ctypes.c_size_t]
    L.fk_server_resident_evict.argtypes = [P, UL]
    L.fk_server_submit.argtypes = [P, ctypes.POINTER(GppRequest), ctypes.POINTER(UL)]
    L.fk_server_wait.argtypes = [P, UL, D, ctypes.POINTER(D)]
    L.fk_server_stats.argtypes = [P, ctypes.POINTER(ServerInfo)]
    L.fk_server_cancel.argtypes = [P, UL]
    L.fk_server_tune.argtypes = [P, I, I, I, I, U, ctypes.POINTER(I)]
    L.fk_set_profiling.argtypes = [P, I]
    L.fk_last_timings.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
    L.fk_last_launches.argtypes = [P]
    L.fk_last_kernel_time.restype = I
    L.fk_last_kernel_time.argtypes = [P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)]
    L.fk_last_transfer.argtypes = [P, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong)]
    L.fk_set_wait_limit.argtypes = [P, ctypes.c_longlong]
    L.fk_selftest_timeout.argtypes = [P, ctypes.c_longlong]
    L.fk_set_error_estimate.argtypes = [P, I]
    L.fk_gpp_error_estimate.argtypes = [P, ctypes.POINTER(D)]
    L.fk_wait_error_status.argtypes = [I, ctypes.c_char_p, ctypes.c_size_t]
    for name in SYMBOLS:
        f = getattr(L, name)
        if name not in ("fk_strerror", "fk_last_error", "fk_version"):
            f.restype = ctypes.c_int
    _lib = L
    return L
