"""Build the sm_103a CUDA library (libfk_gb300.so) and the drop-in command lines.

Plain nvcc, no CMake: every translation unit is compiled in parallel for
sm_103a only, then linked into one shared library with a C ABI
(include/fk_abi.h).  Outputs stay in this directory (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfk_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                  "-I" + os.path.join(ROOT, "include")]
SOURCES = ["fk_abi.cu", "fk_gpp.cu", "fk_ff.cu", "fk_static.cu", "fk_serve.cu"]
CLIS = {"gppKer": "cli_gppKer.cpp", "gppKer_real": "cli_gppKer_real.cpp", "ffKernel": "cli_ffKernel.cpp"}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfk_gb300.so")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "fk_abi.h"))
    flags = NVFLAGS + list(extra or [])
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        if _stale(obj, [src] + headers):
            jobs.append([nvcc()] + flags + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    for exe, src in CLIS.items():
        srcp = os.path.join(CSRC, src)
        out = os.path.join(HERE, exe)
        if os.path.exists(srcp) and _stale(out, [srcp, LIB]):
            _run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), srcp, "-o", out,
                  "-L" + HERE, "-lfk_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
