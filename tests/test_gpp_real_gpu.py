"""GPU parity tests of the real-valued GPP sum (fk_gpp_real, gppKer_real.cpp)
through the C ABI against the oracle.

The real driver's noflag blocks re-add, for a masked term, the value its
scha[] entry still holds (the last unmasked term at that block offset); the
default follows it, FK_GPP_REAL_ZERO_MASKED counts masked terms as 0.  The
branch-stress cases make the mask false for many elements, so the carried
values matter there.

Tolerances (relative, normwise over each output vector):
  FP64 path  <= 1e-12 against the oracle;
  mixed path <= 1e-6 against the FP64 path, scaled by the rss of the terms.
"""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import mixed_gate, rel

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64, TOLMX = 1e-12, 1e-6
KEYS = ("achtemp", "asxtemp", "acht_n1_loc")

CASES = [
    # (nb, nv, nc, ng, dist, index, wx)
    (64, 2, 2048, 19, "branch", "reference", "stress"),   # every branch, carried values
    (40, 5, 1600, 16, "uniform", "even", "e10"), # three flag passes
    (12, 12, 1100, 9, "branch", "reference", "stress"),   # all bands occupied
    (16, 0, 1031, 9, "branch", "reference", "stress"),    # odd ncouls, no occupied bands
    (130, 2, 4099, 70, "branch", "even", "stress"),   # ragged tiles, odd ncouls
    (1, 1, 64, 3, "branch", "reference", "stress"),       # smallest
    (512, 2, 2048, 64, "uniform", "even", "e10"),
]


def ids(c):
    return "x".join(map(str, c[:4])) + "-" + c[4]


def inputs(fk, case, seed=None):
    nb, nv, nc, ng, dist, index, wx = case
    return fk.inputs.gpp_real_synthetic(nb, nv, nc, ng, seed=seed if seed is not None else nb + nc, dist=dist,
                                        index=index, wx=wx)


def real_scales(p, orc, flags):
    o = orc.gpp_real(p, flags=flags, per_pair=True)
    nc = p["ncouls"]
    g = np.array([nc - 1 if i == nc else (p["indinv"][i] if 0 <= i < nc else -1) for i in p["inv_igp_index"]])
    v = np.where(g >= 0, np.asarray(p["vcoul"])[np.maximum(g, 0)], 0.0)
    t, x = o["sch"] * v[None, :, None], o["ssx"] * v[None, :, None]
    return {"achtemp": np.sqrt((t ** 2).sum(axis=(0, 1))),
            "asxtemp": np.sqrt((x ** 2).sum(axis=(0, 1))) if x.size else np.zeros(3),
            "acht_n1_loc": np.sqrt((t[:, :, 2] ** 2).sum(axis=1))}


@pytest.mark.parametrize("zero_masked", [False, True], ids=["carry", "zero"])
@pytest.mark.parametrize("case", CASES, ids=ids)
def test_real_fp64_matches_oracle(ctx, fk, orc, case, zero_masked):
    p = inputs(fk, case)
    flags = fk.FK_GPP_REAL_ZERO_MASKED if zero_masked else 0
    ref = orc.gpp_real(p, flags=orc.ORC_GPP_REAL_ZERO_MASKED if zero_masked else 0)
    res = ctx.gpp_real(p, "fp64", flags)
    errs = {k: rel(res[k], ref[k]) for k in KEYS if np.max(np.abs(ref[k])) > 0}
    assert all(e <= TOL64 for e in errs.values()), errs


@pytest.mark.parametrize("zero_masked", [False, True], ids=["carry", "zero"])
@pytest.mark.parametrize("case", CASES, ids=ids)
def test_real_mixed_within_1e6(ctx, fk, orc, case, zero_masked):
    p = inputs(fk, case)
    flags = fk.FK_GPP_REAL_ZERO_MASKED if zero_masked else 0
    ref = ctx.gpp_real(p, "fp64", flags)
    res = ctx.gpp_real(p, "mixed", flags)
    scales = real_scales(p, orc, orc.ORC_GPP_REAL_ZERO_MASKED if zero_masked else 0)
    mixed_gate(res, ref, scales, TOLMX)


def real_entries():
    with open(os.path.join(GOLD, "reference_drivers.json")) as f:
        return json.load(f)["gppKer_real"]


@pytest.mark.parametrize("entry", real_entries(), ids=lambda e: "x".join(map(str, e["args"])))
def test_real_matches_driver_prints(ctx, fk, entry):
    p = fk.inputs.gpp_real_reference_init(*entry["args"])
    exact = np.array(entry["achtemp_exact"])
    assert rel(ctx.gpp_real(p, "fp64")["achtemp"], exact) <= TOL64
    assert rel(ctx.gpp_real(p, "mixed")["achtemp"], exact) <= TOLMX
    assert rel(ctx.gpp_real(p, "fp64")["achtemp"], entry["achtemp"]) <= TOL64 + rel(entry["achtemp"], exact)


def test_real_benchmark_size(ctx, fk, orc):
    """512 x 2 x 32768 x 20: FP64 against the oracle, mixed against FP64."""
    p = fk.inputs.gpp_real_synthetic(512, 2, 32768, 20, seed=88, dist="branch", wx="e10")
    r64 = ctx.gpp_real(p, "fp64")
    # every host input is staged whole; the three outputs come back
    sent = sum(np.asarray(p[k]).nbytes for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul",
                                                  "inv_igp_index", "indinv", "wx_array"))
    assert ctx.last_transfer() == (sent, (3 + 3 + 512) * 8)
    ref = orc.gpp_real(p)
    for k in KEYS:
        assert rel(r64[k], ref[k]) <= TOL64, k
    rmx = ctx.gpp_real(p, "mixed")
    for k in ("achtemp", "acht_n1_loc"):
        assert rel(rmx[k], r64[k]) <= TOLMX, k


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_real_device_arrays_in_place_and_staged(ctx, fk, prec):
    """Device aqsntemp used in place (even ncouls, aligned), staged when its
    rows are odd-length or it starts 8 bytes past a 16-byte boundary; device
    and host outputs: all the same bits as host inputs."""
    import torch
    for nc in (1500, 1501):
        nb, nv, ng = 70, 3, 11
        p = fk.inputs.gpp_real_synthetic(nb, nv, nc, ng, seed=nc, dist="branch", wx="stress")
        want = ctx.gpp_real(p, prec)
        d = dict(p)
        for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array", "vcoul", "wx_array"):
            d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.float64)).cuda()
        for k in ("inv_igp_index", "indinv"):
            d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.int32)).cuda()
        out = {k: torch.zeros(n, dtype=torch.float64, device="cuda") for k, n in (("achtemp", 3), ("asxtemp", 3),
                                                                                 ("acht_n1_loc", nb))}
        ctx.gpp_real(d, prec, out=out)
        ctx.synchronize()
        for k in KEYS:
            np.testing.assert_array_equal(out[k].cpu().numpy(), want[k])
        # aqsntemp 8 bytes past a 16-byte boundary
        raw = torch.zeros(nb * nc + 1, dtype=torch.float64, device="cuda")
        raw[1:] = d["aqsntemp"].reshape(-1)
        assert (raw.data_ptr() + 8) % 16 == 8
        P = ctypes.c_void_p
        args = [P(d["aqsmtemp"].data_ptr()), P(raw.data_ptr() + 8)] + [
            P(d[k].data_ptr()) for k in ("I_eps_array", "wtilde_array", "vcoul", "inv_igp_index", "indinv",
                                         "wx_array")]
        got = {k: np.zeros(n) for k, n in (("achtemp", 3), ("asxtemp", 3), ("acht_n1_loc", nb))}
        code = fk.FK_FP64 if prec == "fp64" else fk.FK_MIXED
        st = ctx.lib.fk_gpp_real(ctx.h, nb, nv, nc, ng, *args, code, 0, *[P(got[k].ctypes.data) for k in KEYS])
        assert st == 0, ctx.lib.fk_last_error(ctx.h)
        for k in KEYS:
            np.testing.assert_array_equal(got[k], want[k])


def test_real_rejects_bad_arguments(ctx, fk):
    p = fk.inputs.gpp_real_synthetic(8, 2, 64, 4, seed=1)
    with pytest.raises(fk.FKError) as e:
        ctx.gpp_real(dict(p, nvband=9))
    assert e.value.status == 1
    with pytest.raises(fk.FKError) as e:
        ctx.gpp_real(p, "fp64", fk.FK_GPP_HALF_SUM)
    assert e.value.status == 1
