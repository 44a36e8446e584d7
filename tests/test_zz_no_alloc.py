"""fk_gpp_static: the FP64 GPP sum with its scratch in the library's fixed
device array (no allocation), against fk_gpp's FP64 path on the same inputs.

Tolerance: 1e-12 relative, the FP64 path's bar against the reference.  Each
case runs the fixed-scratch call twice in a row on the same scratch.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu
TOL = 1e-12
OUTS = ("achtemp", "asxtemp", "acht_n1_loc", "achstemp")


def device_inputs(p):
    import torch
    d = {}
    for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.complex128)).cuda()
    for k in ("vcoul", "wx_array"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.float64)).cuda()
    for k in ("inv_igp_index", "indinv"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.int32)).cuda()
    return d


def call_static(lib, d, nb, nv, nc, ng, flags, out, stream=0):
    P = ctypes.c_void_p
    ins = [P(d[k].data_ptr()) if hasattr(d[k], "data_ptr") else P(d[k].ctypes.data)
           for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul", "inv_igp_index", "indinv",
                     "wx_array")]
    outs = [P(out[k].data_ptr()) if out.get(k) is not None else None for k in OUTS]
    return lib.fk_gpp_static(P(stream), nb, nv, nc, ng, *ins, flags, *outs)


CASES = [
    # (nb, nv, nc, ng, dist, wx, flags)
    (512, 2, 32768, 20, "uniform", "e10", 0),            # benchmark size
    (130, 2, 4099, 70, "branch", "stress", 0),                # ragged tiles, every branch
    (33, 5, 1000, 13, "branch", "reference", 0x2),            # three flag passes, achstemp
    (64, 2, 777, 7, "branch", "stress", 0x1),                 # root-driver semantics
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])) + f"-f{c[6]}")
def test_static_scratch_matches_fk_gpp_twice(ctx, fk, case):
    import torch
    nb, nv, nc, ng, dist, wx, flags = case
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=31, dist=dist, wx=wx)
    want = ctx.gpp(p, "fp64", flags)
    d = device_inputs(p)
    lib = fk._native.load()
    stream = torch.cuda.Stream()
    for _ in range(2):
        out = {k: torch.full((n,), complex("nan+nanj"), dtype=torch.complex128, device="cuda")
               for k, n in (("achtemp", 3), ("asxtemp", 3), ("acht_n1_loc", nb), ("achstemp", 1))}
        if not flags & fk.FK_GPP_ACHSTEMP:
            out["achstemp"] = None
        torch.cuda.synchronize()
        st = call_static(lib, d, nb, nv, nc, ng, flags, out, stream.cuda_stream)
        assert st == fk._native.FK_OK, lib.fk_strerror(st)
        stream.synchronize()
        for k in OUTS:
            if out[k] is not None:
                assert rel(out[k].cpu().numpy(), want[k]) <= TOL, k


def test_static_scratch_host_outputs(ctx, fk):
    nb, nv, nc, ng = 96, 2, 2000, 10
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=32, dist="branch", wx="stress")
    want = ctx.gpp(p, "fp64")
    d = device_inputs(p)
    lib = fk._native.load()
    got = {"achtemp": np.zeros(3, np.complex128), "asxtemp": np.zeros(3, np.complex128),
           "acht_n1_loc": np.zeros(nb, np.complex128)}
    P = ctypes.c_void_p
    ins = [P(d[k].data_ptr()) for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul",
                                        "inv_igp_index", "indinv", "wx_array")]
    st = lib.fk_gpp_static(None, nb, nv, nc, ng, *ins, 0, *[P(got[k].ctypes.data) for k in OUTS[:3]], None)
    assert st == fk._native.FK_OK
    for k in got:
        assert rel(got[k], want[k]) <= TOL, k


def test_static_scratch_rejects_what_it_cannot_hold(ctx, fk):
    """48*ngpown*ncouls bytes above the 64 MiB array: FK_ENOMEM before any
    work is queued; host input arrays: FK_EINVAL (staging them would need
    memory).  The inputs are full-size device arrays all the same."""
    import torch
    nb, nv, nc, ng = 64, 2, 32768, 64
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=33)
    d = device_inputs(p)
    lib = fk._native.load()
    out = {"achtemp": torch.zeros(3, dtype=torch.complex128, device="cuda"),
           "asxtemp": torch.zeros(3, dtype=torch.complex128, device="cuda"), "acht_n1_loc": None, "achstemp": None}
    assert 48 * ng * nc > 64 << 20
    assert call_static(lib, d, nb, nv, nc, ng, 0, out) == fk._native.FK_ENOMEM
    q = fk.inputs.gpp_synthetic(8, 2, 64, 4, seed=34)
    h = {k: np.ascontiguousarray(v) for k, v in q.items() if isinstance(v, np.ndarray)}
    h["inv_igp_index"] = np.ascontiguousarray(q["inv_igp_index"], np.int32)
    h["indinv"] = np.ascontiguousarray(q["indinv"], np.int32)
    assert call_static(lib, h, 8, 2, 64, 4, 0, out) == fk._native.FK_EINVAL


def test_static_calls_allocate_no_device_memory(ctx, fk):
    """The property the entry point exists for: after a first call (which may
    load the library's scratch array onto the GPU), further calls -- device
    and host outputs, with and without achstemp -- leave the device's free
    memory unchanged."""
    import torch
    nb, nv, nc, ng = 128, 2, 4096, 24
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=35, dist="branch", wx="stress")
    d = device_inputs(p)
    lib = fk._native.load()
    stream = torch.cuda.Stream()
    dev_out = {k: torch.zeros(n, dtype=torch.complex128, device="cuda")
               for k, n in (("achtemp", 3), ("asxtemp", 3), ("acht_n1_loc", nb), ("achstemp", 1))}
    host_out = {"achtemp": np.zeros(3, np.complex128), "asxtemp": np.zeros(3, np.complex128),
                "acht_n1_loc": np.zeros(nb, np.complex128), "achstemp": np.zeros(1, np.complex128)}
    P = ctypes.c_void_p
    ins = [P(d[k].data_ptr()) for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul",
                                        "inv_igp_index", "indinv", "wx_array")]
    assert call_static(lib, d, nb, nv, nc, ng, 0, dev_out, stream.cuda_stream) == fk._native.FK_OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for flags in (0, fk.FK_GPP_ACHSTEMP):
        for _ in range(2):
            o = dict(dev_out)
            if not flags:
                o["achstemp"] = None
            assert call_static(lib, d, nb, nv, nc, ng, flags, o, stream.cuda_stream) == fk._native.FK_OK
            ho = [P(host_out[k].ctypes.data) for k in OUTS[:3]] + [P(host_out["achstemp"].ctypes.data) if flags else None]
            assert lib.fk_gpp_static(P(stream.cuda_stream), nb, nv, nc, ng, *ins, flags, *ho) == fk._native.FK_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    want = ctx.gpp(p, "fp64", fk.FK_GPP_ACHSTEMP)
    for k in OUTS:
        assert rel(host_out[k], want[k]) <= TOL, k
