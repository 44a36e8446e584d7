"""CPU test of the request server's device-block bookkeeping (fk::FirstFit in
csrc/fk_firstfit.h): firstfit_check.cpp drives it with seeded random
allocations and releases against a model of the block (first-fit offsets,
no overlap, in-use and peak bytes, coalesced free ranges, the whole block
free again at the end)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_first_fit_bookkeeping(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "firstfit_check")
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-Wall", "-Werror",
                           "-I", os.path.join(ROOT, "fortkernels-_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "firstfit_check.cpp"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
