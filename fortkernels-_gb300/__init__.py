"""fortkernels_gb300 -- GB300 (sm_103a) GPP and FF self-energy kernels.

Python face of the C ABI in include/fk_abi.h.  The two entry points mirror
the reference mini-apps' hot paths and take their arrays in the reference
layouts:

* :func:`gppKer`   -- the GPP sum of BGW-Kernels/gppKer.cpp:303-439
                      (outputs achtemp[3], asxtemp[3], acht_n1_loc, achstemp)
* :func:`ffKernel` -- the FF kernels of FFKer_cori/ffKernel.cpp:480-503
                      (outputs achsDtemp, asxDtemp, achDtemp, achDtemp_cor,
                      ach2Dtemp, schDt_matrix)

Arrays may be numpy arrays (host memory; staged by the library) or torch
CUDA tensors (device memory; used in place).  All compute runs in the CUDA
library; nothing here computes results on the CPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._native import (FK_FF_PHYSICS, FK_FF_SCHDT_GEMM, FK_FF_SPLIT_ACHD, FK_FP64, FK_GPP_ACHSTEMP,
                      FK_GPP_HALF_SUM, FK_GPP_PHYSICS, FK_GPP_REAL_ZERO_MASKED, FK_GPP_ROOT_QUIRKS, FK_MIXED, FKError)

__all__ = ["Context", "Server", "gppKer", "ffKernel", "FKError", "FK_FP64", "FK_MIXED", "FK_GPP_ROOT_QUIRKS",
           "FK_GPP_ACHSTEMP", "FK_GPP_HALF_SUM", "FK_GPP_PHYSICS", "FK_GPP_REAL_ZERO_MASKED", "FK_FF_SCHDT_GEMM", "FK_FF_PHYSICS", "FK_FF_SPLIT_ACHD", "precision_code"]


def precision_code(p) -> int:
    if p in (FK_FP64, "fp64", "FP64", None):
        return FK_FP64
    if p in (FK_MIXED, "mixed", "MIXED"):
        return FK_MIXED
    raise ValueError(f"unknown precision {p!r}")


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _arg(x, kind: str, n: int, name: str):
    """(pointer, keepalive) for an input array of n elements of `kind`
    ('c128', 'f64', 'i32').  numpy arrays are converted to the exact dtype and
    made contiguous; torch tensors must already be contiguous with that dtype."""
    if _is_torch(x):
        import torch
        want = {"c128": torch.complex128, "f64": torch.float64, "i32": torch.int32}[kind]
        if x.dtype != want or not x.is_contiguous() or x.numel() < n:
            raise ValueError(f"{name}: need a contiguous {want} tensor with >= {n} elements")
        return ctypes.c_void_p(x.data_ptr()), x
    dt = {"c128": np.complex128, "f64": np.float64, "i32": np.int32}[kind]
    a = np.ascontiguousarray(x, dtype=dt)
    if a.size < n:
        raise ValueError(f"{name}: need >= {n} elements, got {a.size}")
    return ctypes.c_void_p(a.ctypes.data), a


class Context:
    """A CUDA context handle of the library (one device, one stream)."""

    def __init__(self, device: int = 0):
        self.lib = _native.load()
        h = ctypes.c_void_p()
        self._check(self.lib.fk_create(device, ctypes.byref(h)), None)
        self.h = h
        self.device = device

    def _check(self, st: int, h):
        if st != _native.FK_OK:
            detail = self.lib.fk_last_error(h).decode() if h is not None else ""
            raise FKError(st, f"{self.lib.fk_strerror(st).decode()}: {detail}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.fk_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int | None):
        self._check(self.lib.fk_set_stream(self.h, ctypes.c_void_p(stream_ptr or 0)), self.h)

    def synchronize(self):
        self._check(self.lib.fk_synchronize(self.h), self.h)

    def reserve(self, nbytes: int):
        self._check(self.lib.fk_reserve(self.h, ctypes.c_size_t(nbytes)), self.h)

    def set_profiling(self, on: bool):
        self._check(self.lib.fk_set_profiling(self.h, int(bool(on))), self.h)

    def last_timings(self):
        ms = (ctypes.c_float * 4)()
        self._check(self.lib.fk_last_timings(self.h, ms), self.h)
        return list(ms)

    def last_launches(self) -> int:
        return int(self.lib.fk_last_launches(self.h))

    def last_kernel_time(self):
        """(milliseconds, launches) of the dominant kernel in the last profiled call."""
        ms, n = ctypes.c_float(), ctypes.c_int()
        self._check(self.lib.fk_last_kernel_time(self.h, ctypes.byref(ms), ctypes.byref(n)), self.h)
        return float(ms.value), int(n.value)

    def set_wait_limit(self, cycles: int):
        """Bound (SM clock cycles) of the tensor-core kernels' waits; negative: the default.
        Lowering it is a test hook for the timeout path."""
        self._check(self.lib.fk_set_wait_limit(self.h, int(cycles)), self.h)

    def set_error_estimate(self, enable: bool = True):
        """Make later mixed gpp calls also compute an a-priori error estimate
        (one more pass over aqsntemp); read it with gpp_error_estimate()."""
        self._check(self.lib.fk_set_error_estimate(self.h, 1 if enable else 0), self.h)

    def gpp_error_estimate(self) -> dict:
        """Estimated absolute error of the last mixed gpp call's outputs:
        {"achtemp": max over iw, "asxtemp": max over iw, "acht_n1_loc": max over bands}."""
        v = (ctypes.c_double * 3)()
        self._check(self.lib.fk_gpp_error_estimate(self.h, v), self.h)
        return {"achtemp": v[0], "asxtemp": v[1], "acht_n1_loc": v[2]}

    def selftest_timeout(self, cycles: int) -> int:
        """Status of a one-warp kernel whose bounded wait on a barrier nothing
        arrives on gives up after `cycles` cycles (FK_ETIMEOUT expected)."""
        return int(self.lib.fk_selftest_timeout(self.h, int(cycles)))

    def last_transfer(self):
        """(host-to-device, device-to-host) bytes of the last gpp / gpp_real / ff call."""
        h, d = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        self._check(self.lib.fk_last_transfer(self.h, ctypes.byref(h), ctypes.byref(d)), self.h)
        return int(h.value), int(d.value)

    # ------------------------------------------------------------------ GPP
    def gpp(self, p: dict, precision="fp64", flags: int = 0, out=None) -> dict:
        """GPP sum on the input dict (keys as in fortkernels_gb300.inputs)."""
        nb, nv, nc, ng = int(p["number_bands"]), int(p["nvband"]), int(p["ncouls"]), int(p["ngpown"])
        keep = []

        def a(key, kind, n):
            ptr, k = _arg(p[key], kind, n, key)
            keep.append(k)
            return ptr

        args = [a("aqsmtemp", "c128", nb * nc), a("aqsntemp", "c128", nb * nc),
                a("I_eps_array", "c128", ng * nc), a("wtilde_array", "c128", ng * nc),
                a("vcoul", "f64", nc), a("inv_igp_index", "i32", ng), a("indinv", "i32", nc),
                a("wx_array", "f64", 3)]
        if out is None:
            out = {"achtemp": np.zeros(3, np.complex128), "asxtemp": np.zeros(3, np.complex128),
                   "acht_n1_loc": np.zeros(nb, np.complex128), "achstemp": np.zeros(1, np.complex128)}
        optr = [ctypes.c_void_p(_data_ptr(out[k])) if out.get(k) is not None else None
                for k in ("achtemp", "asxtemp", "acht_n1_loc", "achstemp")]
        st = self.lib.fk_gpp(self.h, nb, nv, nc, ng, *args, precision_code(precision), flags, *optr)
        self._check(st, self.h)
        return out

    def gpp_real(self, p: dict, precision="fp64", flags: int = 0, out=None) -> dict:
        """Real-valued GPP sum (gppKer_real.cpp) on a dict of float64 arrays."""
        nb, nv, nc, ng = int(p["number_bands"]), int(p["nvband"]), int(p["ncouls"]), int(p["ngpown"])
        keep = []

        def a(key, kind, n):
            ptr, k = _arg(p[key], kind, n, key)
            keep.append(k)
            return ptr

        args = [a("aqsmtemp", "f64", nb * nc), a("aqsntemp", "f64", nb * nc), a("I_eps_array", "f64", ng * nc),
                a("wtilde_array", "f64", ng * nc), a("vcoul", "f64", nc), a("inv_igp_index", "i32", ng),
                a("indinv", "i32", nc), a("wx_array", "f64", 3)]
        if out is None:
            out = {"achtemp": np.zeros(3), "asxtemp": np.zeros(3), "acht_n1_loc": np.zeros(nb)}
        optr = [ctypes.c_void_p(_data_ptr(out[k])) if out.get(k) is not None else None
                for k in ("achtemp", "asxtemp", "acht_n1_loc")]
        st = self.lib.fk_gpp_real(self.h, nb, nv, nc, ng, *args, precision_code(precision), flags, *optr)
        self._check(st, self.h)
        return out

    # ------------------------------------------------------------------- FF
    def ff(self, p: dict, precision="fp64", flags: int = 0, out=None) -> dict:
        nb, nv, nc, ng = int(p["number_bands"]), int(p["nvband"]), int(p["ncouls"]), int(p["ngpown"])
        nf, ne = int(p["nFreq"]), int(p["nfreqeval"])
        keep = []

        def a(key, kind, n):
            ptr, k = _arg(p[key], kind, n, key)
            keep.append(k)
            return ptr

        args = [a("aqsmtemp", "c128", nb * nc), a("aqsntemp", "c128", nb * nc),
                a("I_epsR_array", "c128", nf * ng * nc), a("I_epsA_array", "c128", nf * ng * nc),
                a("vcoul", "f64", nc), a("inv_igp_index", "i32", ng), a("indinv", "i32", nc),
                a("ekq", "f64", nb), a("dFreqGrid", "f64", nf), a("dFreqBrd", "c128", nf), a("pref", "f64", nf)]
        if out is None:
            out = {"achsDtemp": np.zeros(1, np.complex128), "asxDtemp": np.zeros(ne, np.complex128),
                   "achDtemp": np.zeros(ne, np.complex128), "achDtemp_cor": np.zeros(ne, np.complex128),
                   "ach2Dtemp": np.zeros(ne, np.complex128), "schDt_matrix": np.zeros((nb, nf), np.complex128)}
        optr = [ctypes.c_void_p(_data_ptr(out[k])) if out.get(k) is not None else None
                for k in ("achsDtemp", "asxDtemp", "achDtemp", "achDtemp_cor", "ach2Dtemp", "schDt_matrix")]
        st = self.lib.fk_ff(self.h, nb, nv, nc, ng, nf, ne, *args, float(p["pref_zb"]), float(p["freqevalmin"]),
                            float(p["freqevalstep"]), float(p.get("occ", 1.0)), precision_code(precision), flags,
                            *optr)
        self._check(st, self.h)
        return out


class Server:
    """GPP request server (fk_server_* of include/fk_abi.h): requests of any
    size are submitted as they arrive and run in fused steps on one GPU.
    Input arrays (numpy or torch) are kept referenced until the request is
    waited for."""

    def __init__(self, device: int = 0, hbm_bytes: int = 8 << 30, max_active: int = 16, step_stages: int = 0):
        self.lib = _native.load()
        cfg = _native.ServerConfig(hbm_bytes, max_active, step_stages)
        h = ctypes.c_void_p()
        st = self.lib.fk_server_create(device, ctypes.byref(cfg), ctypes.byref(h))
        if st != _native.FK_OK:
            raise FKError(st, f"fk_server_create: {self.lib.fk_strerror(st).decode()}")
        self.h = h
        self._pending = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.fk_server_destroy(self.h)
            self.h = None
            self._pending.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != _native.FK_OK:
            raise FKError(st, f"{what}: {self.lib.fk_strerror(st).decode()}")

    def resident_put(self, key: int, array):
        ptr, keep = _arg(array, "c128", 1, "resident array")
        n = keep.numel() * keep.element_size() if _is_torch(keep) else keep.nbytes
        self._check(self.lib.fk_server_resident_put(self.h, key, ptr, n), "fk_server_resident_put")

    def resident_evict(self, key: int):
        self._check(self.lib.fk_server_resident_evict(self.h, key), "fk_server_resident_evict")

    def submit(self, p: dict, flags: int = 0, eps_key=None, wtilde_key=None, out=None) -> int:
        """Queue a GPP request (keys of fortkernels_gb300.inputs); returns its ticket.
        eps_key / wtilde_key name resident arrays instead of p's I_eps_array /
        wtilde_array."""
        nb, nv, nc, ng = int(p["number_bands"]), int(p["nvband"]), int(p["ncouls"]), int(p["ngpown"])
        keep = []

        def a(key, kind, n):
            ptr, k = _arg(p[key], kind, n, key)
            keep.append(k)
            return ptr

        q = _native.GppRequest()
        q.number_bands, q.nvband, q.ncouls, q.ngpown = nb, nv, nc, ng
        q.aqsmtemp, q.aqsntemp = a("aqsmtemp", "c128", nb * nc), a("aqsntemp", "c128", nb * nc)
        q.I_eps_array = None if eps_key is not None else a("I_eps_array", "c128", ng * nc)
        q.wtilde_array = None if wtilde_key is not None else a("wtilde_array", "c128", ng * nc)
        q.eps_key = eps_key or 0
        q.wtilde_key = wtilde_key or 0
        q.vcoul, q.inv_igp_index = a("vcoul", "f64", nc), a("inv_igp_index", "i32", ng)
        q.indinv, q.wx_array = a("indinv", "i32", nc), a("wx_array", "f64", 3)
        q.flags = flags
        if out is None:
            out = {"achtemp": np.zeros(3, np.complex128), "asxtemp": np.zeros(3, np.complex128),
                   "acht_n1_loc": np.zeros(nb, np.complex128)}
        q.achtemp, q.asxtemp = _data_ptr(out["achtemp"]), _data_ptr(out["asxtemp"])
        q.acht_n1_loc = _data_ptr(out["acht_n1_loc"]) if out.get("acht_n1_loc") is not None else None
        t = ctypes.c_ulonglong()
        self._check(self.lib.fk_server_submit(self.h, ctypes.byref(q), ctypes.byref(t)), "fk_server_submit")
        self._pending[t.value] = (keep, out)
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0):
        """(outputs, latency in seconds) of a submitted request."""
        lat = ctypes.c_double()
        st = self.lib.fk_server_wait(self.h, ticket, timeout, ctypes.byref(lat))
        keep, out = self._pending.get(ticket, (None, None))
        if st != _native.FK_EBUSY:
            self._pending.pop(ticket, None)
        self._check(st, "fk_server_wait")
        return out, lat.value

    def cancel(self, ticket: int) -> int:
        """Cancel a request still waiting for admission; returns the status
        (FK_OK: cancelled, its wait gives FK_ECANCELED; FK_EBUSY: already admitted)."""
        return int(self.lib.fk_server_cancel(self.h, ticket))

    def tune(self, number_bands: int, nvband: int, ncouls: int, ngpown: int, flags: int = 0) -> int:
        """Autotune the plan of a request shape (server idle); returns the chosen k-slice count."""
        ks = ctypes.c_int()
        self._check(self.lib.fk_server_tune(self.h, number_bands, nvband, ncouls, ngpown, flags, ctypes.byref(ks)),
                    "fk_server_tune")
        return ks.value

    def stats(self) -> dict:
        i = _native.ServerInfo()
        self._check(self.lib.fk_server_stats(self.h, ctypes.byref(i)), "fk_server_stats")
        return {f: getattr(i, f) for f, _ in _native.ServerInfo._fields_}


def _data_ptr(x) -> int:
    return x.data_ptr() if _is_torch(x) else x.ctypes.data


_default_ctx = None


def _ctx() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def gppKer(p: dict, precision="fp64", flags: int = 0) -> dict:
    """GPP self-energy sum (BGW-Kernels/gppKer.cpp:303-439) on device 0."""
    return _ctx().gpp(p, precision, flags)


def ffKernel(p: dict, precision="fp64", flags: int = 0) -> dict:
    """FF full-frequency kernels (FFKer_cori/ffKernel.cpp:480-503) on device 0."""
    return _ctx().ff(p, precision, flags)
