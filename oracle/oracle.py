"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.  It loads ``oracle/liboracle.so`` (the C restatement of the
reference loops, ``fk_oracle.c``) and, when the reference tree was present at
build time, runs the binaries under ``oracle/_ref/`` (the unmodified reference
drivers and the harnesses that call the reference's own solver functions).
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

ORC_GPP_ROOT_QUIRKS = 0x1
ORC_GPP_ACHSTEMP = 0x2
ORC_GPP_HALF_SUM = 0x4
ORC_GPP_PHYSICS = 0x8
ORC_GPP_REAL_ZERO_MASKED = 0x10
ORC_FF_SCHDT_GEMM = 0x1
ORC_FF_PHYSICS = 0x2
ORC_FF_SPLIT_ACHD = 0x4

_lib = None


def build(quiet: bool = True) -> None:
    """Compile liboracle.so (and oracle/_ref/ when the reference sources are at hand:
    FK_REFERENCE_DIR, or their copy in oracle/_ref/src/)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"], stdout=out)
    ref = os.environ.get("FK_REFERENCE_DIR")
    if (ref and os.path.isdir(ref)) or os.path.isdir(os.path.join(REF_DIR, "src")):
        subprocess.check_call(["make", "-s", "-j8", "-C", HERE, "ref"], stdout=out)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_gpp.restype = ctypes.c_int
        L.orc_gpp.argtypes = [ctypes.c_int] * 4 + [dp] * 5 + [ip, ip, ctypes.c_int, dp, ctypes.c_uint, ctypes.c_int] + [dp] * 6
        L.orc_gpp_real.restype = ctypes.c_int
        L.orc_gpp_real.argtypes = ([ctypes.c_int] * 4 + [dp] * 5 + [ip, ip, ctypes.c_int, dp, ctypes.c_uint,
                                   ctypes.c_int] + [dp] * 5)
        L.orc_ff.restype = ctypes.c_int
        L.orc_ff.argtypes = ([ctypes.c_int] * 6 + [dp] * 5 + [ip, ip] + [dp] * 4 +
                             [ctypes.c_double] * 4 + [ctypes.c_uint, ctypes.c_int] + [dp] * 6)
        L.orc_ff_compute_fact.restype = None
        L.orc_ff_compute_fact.argtypes = [ctypes.c_double, ctypes.c_int, dp, dp, dp, ip, ctypes.c_int, ctypes.c_int]
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _c(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def gpp(p: dict, flags: int = 0, nthreads: int = 0, per_pair: bool = False) -> dict:
    """Oracle GPP on the input dict produced by fortkernels_gb300.inputs."""
    nb, nv, nc, ng = p["number_bands"], p["nvband"], p["ncouls"], p["ngpown"]
    aqsm, aqsn = _c(p["aqsmtemp"]), _c(p["aqsntemp"])
    eps, wt = _c(p["I_eps_array"]), _c(p["wtilde_array"])
    vcoul = np.ascontiguousarray(p["vcoul"], dtype=np.float64)
    inv = np.ascontiguousarray(p["inv_igp_index"], dtype=np.int32)
    indinv = np.ascontiguousarray(p["indinv"], dtype=np.int32)
    wx = np.ascontiguousarray(p["wx_array"], dtype=np.float64)
    ach = np.zeros(3, np.complex128)
    asx = np.zeros(3, np.complex128)
    n1loc = np.zeros(nb, np.complex128)
    achs = np.zeros(1, np.complex128)
    sch = np.zeros((nb, ng, 3), np.complex128) if per_pair else None
    ssx = np.zeros((max(nv, 1), ng, 3), np.complex128) if per_pair else None
    rc = lib().orc_gpp(nb, nv, nc, ng, _dp(aqsm.view(np.float64)), _dp(aqsn.view(np.float64)),
                       _dp(eps.view(np.float64)), _dp(wt.view(np.float64)), _dp(vcoul), _ip(inv), _ip(indinv),
                       len(indinv), _dp(wx), flags, nthreads, _dp(ach.view(np.float64)), _dp(asx.view(np.float64)),
                       _dp(n1loc.view(np.float64)), _dp(achs.view(np.float64)),
                       None if sch is None else _dp(sch.view(np.float64)),
                       None if ssx is None else _dp(ssx.view(np.float64)))
    if rc != 0:
        raise ValueError(f"orc_gpp rc={rc}")
    out = {"achtemp": ach, "asxtemp": asx, "acht_n1_loc": n1loc, "achstemp": achs[0]}
    if per_pair:
        out["sch"], out["ssx"] = sch, ssx[:nv]
    return out


def gpp_real(p: dict, flags: int = 0, nthreads: int = 0, per_pair: bool = False) -> dict:
    """Oracle real-valued GPP (gppKer_real.cpp) on a dict of real arrays."""
    nb, nv, nc, ng = p["number_bands"], p["nvband"], p["ncouls"], p["ngpown"]
    f = {k: np.ascontiguousarray(p[k], dtype=np.float64)
         for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul", "wx_array")}
    inv = np.ascontiguousarray(p["inv_igp_index"], dtype=np.int32)
    indinv = np.ascontiguousarray(p["indinv"], dtype=np.int32)
    ach, asx, n1loc = np.zeros(3), np.zeros(3), np.zeros(nb)
    sch = np.zeros((nb, ng, 3)) if per_pair else None
    ssx = np.zeros((max(nv, 1), ng, 3)) if per_pair else None
    rc = lib().orc_gpp_real(nb, nv, nc, ng, _dp(f["aqsmtemp"]), _dp(f["aqsntemp"]), _dp(f["I_eps_array"]),
                            _dp(f["wtilde_array"]), _dp(f["vcoul"]), _ip(inv), _ip(indinv), len(indinv),
                            _dp(f["wx_array"]), flags, nthreads, _dp(ach), _dp(asx), _dp(n1loc), _dp(sch), _dp(ssx))
    if rc != 0:
        raise ValueError(f"orc_gpp_real rc={rc}")
    out = {"achtemp": ach, "asxtemp": asx, "acht_n1_loc": n1loc}
    if per_pair:
        out["sch"], out["ssx"] = sch, ssx[:nv]
    return out


def ff(p: dict, flags: int = 0, nthreads: int = 0) -> dict:
    """Oracle FF on the input dict produced by fortkernels_gb300.inputs."""
    nb, nv, nc, ng = p["number_bands"], p["nvband"], p["ncouls"], p["ngpown"]
    nf, ne = p["nFreq"], p["nfreqeval"]
    a = {k: _c(p[k]) for k in ("aqsmtemp", "aqsntemp", "I_epsR_array", "I_epsA_array", "dFreqBrd")}
    d = {k: np.ascontiguousarray(p[k], dtype=np.float64) for k in ("vcoul", "ekq", "dFreqGrid", "pref")}
    inv = np.ascontiguousarray(p["inv_igp_index"], dtype=np.int32)
    indinv = np.ascontiguousarray(p["indinv"], dtype=np.int32)
    achs = np.zeros(1, np.complex128)
    asx = np.zeros(ne, np.complex128)
    achd = np.zeros(ne, np.complex128)
    cor = np.zeros(ne, np.complex128)
    a2 = np.zeros(ne, np.complex128)
    schdt = np.zeros((nb, nf), np.complex128)
    v = lambda x: _dp(x.view(np.float64))
    rc = lib().orc_ff(nb, nv, nc, ng, nf, ne, v(a["aqsmtemp"]), v(a["aqsntemp"]), v(a["I_epsR_array"]),
                      v(a["I_epsA_array"]), _dp(d["vcoul"]), _ip(inv), _ip(indinv), _dp(d["ekq"]),
                      _dp(d["dFreqGrid"]), v(a["dFreqBrd"]), _dp(d["pref"]), float(p["pref_zb"]),
                      float(p["freqevalmin"]), float(p["freqevalstep"]), float(p.get("occ", 1.0)), flags, nthreads,
                      v(achs), v(asx), v(achd), v(cor), v(a2), v(schdt))
    if rc != 0:
        raise ValueError(f"orc_ff rc={rc}")
    return {"achsDtemp": achs[0], "asxDtemp": asx, "achDtemp": achd, "achDtemp_cor": cor,
            "ach2Dtemp": a2, "schDt_matrix": schdt}


def compute_fact(wx: float, grid, loop: int, flag_occ: bool):
    g = np.ascontiguousarray(grid, dtype=np.float64)
    f1 = ctypes.c_double(0.0)
    f2 = ctypes.c_double(0.0)
    fi = ctypes.c_int(0)
    lib().orc_ff_compute_fact(wx, len(g), _dp(g), ctypes.byref(f1), ctypes.byref(f2), ctypes.byref(fi),
                              loop, int(flag_occ))
    return f1.value, f2.value, fi.value


# ---------------------------------------------------------------- reference

def have_ref() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "ref_harness_gpp"))


_CPLX = re.compile(r"\(\s*([-+0-9.eEinfa]+)\s*,\s*([-+0-9.eEinfa]+)\s*\)")
_REAL = re.compile(r"\s*([-+]?[0-9.]+(?:[eE][-+]?[0-9]+)?)\s*$")


def run_ref_driver(name: str, args, threads: int = 8) -> dict:
    """Run an unmodified reference driver from oracle/_ref and parse its output."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = subprocess.run([os.path.join(REF_DIR, name)] + [str(a) for a in args], env=env,
                         capture_output=True, text=True, check=True).stdout
    res = {"stdout": out}
    for line in out.splitlines():
        m = re.match(r"\s*(\w+)(\[(\d+)\])?\s*=\s*(.*)$", line)
        if not m:
            continue
        c = _CPLX.search(m.group(4))
        key = m.group(1) + (f"[{m.group(3)}]" if m.group(2) else "")
        if c:
            res[key] = complex(float(c.group(1)), float(c.group(2)))
            continue
        r = _REAL.match(m.group(4))  # the real-valued driver prints plain numbers
        if r:
            res[key] = float(r.group(1))
    t = re.search(r"Chrono Time Taken \*+= ([0-9.eE+-]+)", out)
    if t:
        res["seconds"] = float(t.group(1))
    return res


def ref_gpp_pairs(p: dict, igp: np.ndarray, gppsum: int = 0) -> dict:
    """Per-(n1, my_igp, iw) sch/ssx from the reference's own solver functions
    (gppsum=1: gppKerSeq.cpp's half-sum mode)."""
    nb, nv, nc, ng = p["number_bands"], p["nvband"], p["ncouls"], p["ngpown"]
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array"):
                f.write(_c(p[k]).tobytes())
            f.write(np.ascontiguousarray(p["wx_array"], np.float64).tobytes())
            f.write(np.ascontiguousarray(igp, np.int32).tobytes())
        subprocess.run([os.path.join(REF_DIR, "ref_harness_gpp")] + [str(x) for x in (nb, nv, nc, ng, fin, fout)] +
                       ([str(gppsum)] if gppsum else []),
                       check=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
        raw = np.fromfile(fout, dtype=np.complex128)
    sch = raw[: nb * ng * 3].reshape(nb, ng, 3)
    ssx = raw[nb * ng * 3:].reshape(nv, ng, 3) if nv > 0 else np.zeros((0, ng, 3), np.complex128)
    return {"sch": sch, "ssx": ssx}


def ref_gpp_real_pairs(p: dict, igp: np.ndarray) -> dict:
    """Per-(n1 < nvband, my_igp, iw) sch/ssx of the real-valued driver's own
    flagOCC_solver (gppKer_real.cpp)."""
    nb, nv, nc, ng = p["number_bands"], p["nvband"], p["ncouls"], p["ngpown"]
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "wx_array"):
                f.write(np.ascontiguousarray(p[k], np.float64).tobytes())
            f.write(np.ascontiguousarray(igp, np.int32).tobytes())
        subprocess.run([os.path.join(REF_DIR, "ref_harness_gpp_real")] + [str(x) for x in (nb, nv, nc, ng, fin, fout)],
                       check=True, env=dict(os.environ, OMP_NUM_THREADS="1"))
        raw = np.fromfile(fout, dtype=np.float64)
    return {"sch": raw[: nv * ng * 3].reshape(nv, ng, 3), "ssx": raw[nv * ng * 3:].reshape(nv, ng, 3)}


def ref_ff(p: dict, schDt=None) -> dict:
    """FF outputs from the reference's own kernels (single thread)."""
    nb, nv, nc, ng = p["number_bands"], p["nvband"], p["ncouls"], p["ngpown"]
    nf, ne = p["nFreq"], p["nfreqeval"]
    if schDt is None:
        schDt = np.zeros((nb, nf), np.complex128)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            for k in ("aqsmtemp", "aqsntemp", "I_epsR_array", "I_epsA_array", "dFreqBrd"):
                f.write(_c(p[k]).tobytes())
            f.write(_c(schDt).tobytes())
            for k in ("vcoul", "ekq", "dFreqGrid", "pref"):
                f.write(np.ascontiguousarray(p[k], np.float64).tobytes())
            f.write(np.array([p["pref_zb"], p["freqevalmin"], p["freqevalstep"], p.get("occ", 1.0)],
                             np.float64).tobytes())
            f.write(np.ascontiguousarray(p["inv_igp_index"], np.int32).tobytes())
            f.write(np.ascontiguousarray(p["indinv"], np.int32).tobytes())
        subprocess.run([os.path.join(REF_DIR, "ref_harness_ff")] + [str(x) for x in (nb, nv, nc, ng, nf, ne, fin, fout)],
                       check=True, env=dict(os.environ, OMP_NUM_THREADS="1"))
        raw = np.fromfile(fout, dtype=np.complex128)
    return {"achsDtemp": raw[0], "asxDtemp": raw[1:1 + ne], "achDtemp_cor": raw[1 + ne:1 + 2 * ne],
            "ach2Dtemp": raw[1 + 2 * ne:1 + 3 * ne]}
