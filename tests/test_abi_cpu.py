"""CPU tests of the boundary: the C-ABI library loads, exports every symbol
include/fk_abi.h declares, and rejects bad calls without touching a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fk_abi.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(fk_\w+)\s*\(", src, re.M)))


def test_header_declares_the_entry_points():
    names = declared()
    for n in ("fk_create", "fk_destroy", "fk_gpp", "fk_ff", "fk_strerror", "fk_last_timings"):
        assert n in names


def test_library_exports_every_declared_symbol(fk):
    lib = fk._native.load()
    path = fk._native.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (fk_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    for n in declared():
        assert hasattr(lib, n)
    assert set(fk._native.SYMBOLS) == set(declared())


def test_abi_has_no_torch_dependency(fk):
    out = subprocess.run(["ldd", fk._native.LIB_PATH], capture_output=True, text=True).stdout
    assert "torch" not in out and "c10" not in out


def test_version_and_strerror(fk):
    lib = fk._native.load()
    assert lib.fk_version().decode().startswith("fk_gb300")
    for code in range(8):
        assert lib.fk_strerror(code).decode()
    assert lib.fk_strerror(99).decode() == "unknown status"


def test_null_context_is_rejected(fk):
    lib = fk._native.load()
    z = ctypes.c_void_p(0)
    assert lib.fk_gpp(z, 1, 0, 1, 1, *([z] * 8), 0, 0, *([z] * 4)) == fk._native.FK_EINVAL
    assert lib.fk_ff(z, 1, 0, 1, 1, 2, 1, *([z] * 11), 0.0, 0.0, 0.5, 1.0, 0, 0, *([z] * 6)) == fk._native.FK_EINVAL
    assert lib.fk_destroy(z) == fk._native.FK_EINVAL
    assert lib.fk_create(0, None) == fk._native.FK_EINVAL
    assert lib.fk_last_launches(z) == -1


def test_create_without_gpu_fails_cleanly(fk):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = fk._native.load()
    h = ctypes.c_void_p()
    assert lib.fk_create(0, ctypes.byref(h)) == fk._native.FK_ECUDA
    with pytest.raises(fk.FKError):
        fk.Context(0)


def test_missing_library_fails_loudly(fk, tmp_path):
    with pytest.raises(fk.FKError):
        fk._native._lib_backup = fk._native._lib
        fk._native._lib = None
        try:
            fk._native.load(str(tmp_path / "nope.so"))
        finally:
            fk._native._lib = fk._native._lib_backup


def test_python_argument_checks(fk):
    import numpy as np
    ptr, keep = fk._arg(np.arange(4), "f64", 4, "x")
    assert keep.dtype == np.float64 and ptr.value == keep.ctypes.data
    with pytest.raises(ValueError):
        fk._arg(np.zeros(2), "c128", 3, "x")
    assert fk.precision_code("mixed") == fk.FK_MIXED and fk.precision_code("fp64") == fk.FK_FP64
    with pytest.raises(ValueError):
        fk.precision_code("fp8")


def test_wait_error_word_maps_to_timeout(fk):
    """The device error word of the tensor-core kernels (set when a bounded
    wait gives up) maps to FK_ETIMEOUT with a message naming the waits; 0 is
    FK_OK.  Host logic only: no GPU."""
    lib = fk._native.load()
    buf = ctypes.create_string_buffer(512)
    assert lib.fk_wait_error_status(0, buf, 512) == fk._native.FK_OK
    assert lib.fk_wait_error_status(0x10, buf, 512) == fk._native.FK_ETIMEOUT
    assert b"epilogue" in buf.value and b"0x10" in buf.value
    assert lib.fk_wait_error_status(0x2 | 0x20 | 0x80, buf, 512) == fk._native.FK_ETIMEOUT
    msg = buf.value.decode()
    assert "operand stage" in msg and "converter" in msg and "last copies" in msg
    assert lib.fk_wait_error_status(0x100, buf, 512) == fk._native.FK_ETIMEOUT
    assert "self-test" in buf.value.decode()
    assert lib.fk_wait_error_status(0x200, buf, 512) == fk._native.FK_ETIMEOUT
    assert "plane conversion" in buf.value.decode() and "unknown" not in buf.value.decode()
    assert lib.fk_wait_error_status(0x400, buf, 512) == fk._native.FK_ETIMEOUT
    assert "-B_im" in buf.value.decode() and "unknown" not in buf.value.decode()
    assert lib.fk_wait_error_status(0x4000, buf, 512) == fk._native.FK_ETIMEOUT
    assert "unknown" in buf.value.decode()
    small = ctypes.create_string_buffer(8)
    assert lib.fk_wait_error_status(0x1, small, 8) == fk._native.FK_ETIMEOUT
    assert len(small.value) == 7  # truncated, NUL-terminated
    assert lib.fk_wait_error_status(0x1, None, 0) == fk._native.FK_ETIMEOUT
