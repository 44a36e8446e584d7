"""GPU parity tests of the GPP path (fk_gpp through the C ABI) against the oracle.

Tolerances (relative, normwise over each output vector):
  FP64 path  <= 1e-12 against the oracle (the reference C++ semantics);
  mixed path <= 1e-6 against the FP64 path and the oracle.
"""
import json
import os

import numpy as np
import pytest

from conftest import gpp_scales, mixed_gate, rel

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64, TOLMX = 1e-12, 1e-6


def check(res, ref, tol, keys=("achtemp", "asxtemp", "acht_n1_loc")):
    errs = {k: rel(res[k], ref[k]) for k in keys}
    assert all(e <= tol for e in errs.values()), errs
    return errs


CASES = [
    # (nb, nv, nc, ng, dist, index, wx)
    (512, 2, 2048, 64, "uniform", "even", "e10"),   # the reference's small CPU-runnable case
    (64, 2, 777, 7, "branch", "reference", "stress"),         # ragged, every branch
    (33, 5, 1000, 13, "branch", "even", "reference"),     # three flag passes
    (16, 0, 640, 9, "uniform", "reference", "reference"),     # no occupied bands
    (12, 12, 300, 4, "branch", "reference", "stress"),        # all bands occupied
    (1, 1, 64, 1, "branch", "even", "stress"),            # smallest
    (130, 2, 4099, 70, "branch", "reference", "stress"),      # tile edges
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])) + "-" + c[4])
def test_gpp_fp64_matches_oracle(ctx, fk, orc, case):
    nb, nv, nc, ng, dist, index, wx = case
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=nb + nc, dist=dist, index=index, wx=wx)
    ref = orc.gpp(p)
    check(ctx.gpp(p, "fp64"), ref, TOL64)


def check_mixed(res, ref, scales, tol=TOLMX):
    return mixed_gate(res, ref, scales, tol)


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])) + "-" + c[4])
def test_gpp_mixed_within_1e6(ctx, fk, orc, case):
    nb, nv, nc, ng, dist, index, wx = case
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=nb + nc, dist=dist, index=index, wx=wx)
    ref = ctx.gpp(p, "fp64")
    check_mixed(ctx.gpp(p, "mixed"), ref, gpp_scales(p, orc))


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpp_root_quirks(ctx, fk, orc, prec):
    p = fk.inputs.gpp_synthetic(40, 3, 900, 9, seed=7, dist="branch", index="reference", wx="stress")
    ref = orc.gpp(p, flags=orc.ORC_GPP_ROOT_QUIRKS)
    res = ctx.gpp(p, prec, fk.FK_GPP_ROOT_QUIRKS)
    if prec == "fp64":
        check(res, ref, TOL64)
    else:
        check_mixed(res, ref, gpp_scales(p, orc, orc.ORC_GPP_ROOT_QUIRKS))


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpp_static_remainder(ctx, fk, orc, prec):
    p = fk.inputs.gpp_synthetic(48, 2, 1024, 16, seed=8, dist="uniform")
    ref = orc.gpp(p, flags=orc.ORC_GPP_ACHSTEMP)
    r = ctx.gpp(p, prec, fk.FK_GPP_ACHSTEMP)
    if prec == "fp64":
        assert rel(r["achstemp"], [ref["achstemp"]]) <= TOL64
        check(r, ref, TOL64)
    else:
        assert rel(r["achstemp"], [ref["achstemp"]]) <= TOLMX
        check_mixed(r, ref, gpp_scales(p, orc))


def golden(name):
    with open(os.path.join(GOLD, "reference_drivers.json")) as f:
        return json.load(f)[name]


def driver_check(res, entry, tol):
    """The driver's printed value carries its own summation error; the exact
    closed form of its constant inputs is the tight target."""
    exact = np.array([complex(*z) for z in entry["achtemp_exact"]])
    printed = np.array([complex(*z) for z in entry["achtemp"]])
    assert rel(res, exact) <= tol
    assert rel(res, printed) <= tol + rel(printed, exact)


@pytest.mark.parametrize("entry", golden("gppKer_bgw"), ids=lambda e: "x".join(map(str, e["args"])))
def test_gpp_matches_reference_driver_prints(ctx, fk, entry):
    p = fk.inputs.gpp_reference_init(*entry["args"])
    driver_check(ctx.gpp(p, "fp64")["achtemp"], entry, TOL64)
    driver_check(ctx.gpp(p, "mixed")["achtemp"], entry, TOLMX)


@pytest.mark.parametrize("entry", golden("gppKer_root"), ids=lambda e: "x".join(map(str, e["args"])))
def test_gpp_matches_root_driver_prints(ctx, fk, entry):
    p = fk.inputs.gpp_reference_init(*entry["args"])
    driver_check(ctx.gpp(p, "fp64", fk.FK_GPP_ROOT_QUIRKS)["achtemp"], entry, TOL64)


def test_gpp_skips_unmapped_columns(ctx, fk, orc):
    p = fk.inputs.gpp_synthetic(20, 2, 500, 8, seed=9, dist="branch", wx="stress")
    p["inv_igp_index"] = p["inv_igp_index"].copy()
    p["inv_igp_index"][[1, 5]] = [-3, 10_000]     # out of range: skipped like the reference
    p["inv_igp_index"][6] = 500                   # == ncouls: clamped to ncouls-1
    ref = orc.gpp(p)
    check(ctx.gpp(p, "fp64"), ref, TOL64)


def test_gpp_device_pointers_equal_host_pointers(ctx, fk):
    import torch
    p = fk.inputs.gpp_synthetic(70, 2, 1500, 11, seed=10, dist="branch", wx="stress")
    host = ctx.gpp(p, "fp64")
    d = dict(p)
    for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k])).cuda()
    for k in ("vcoul", "wx_array"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.float64)).cuda()
    for k in ("inv_igp_index", "indinv"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.int32)).cuda()
    out = {"achtemp": torch.zeros(3, dtype=torch.complex128, device="cuda"),
           "asxtemp": torch.zeros(3, dtype=torch.complex128, device="cuda"),
           "acht_n1_loc": torch.zeros(70, dtype=torch.complex128, device="cuda"),
           "achstemp": None}
    dev = ctx.gpp(d, "fp64", out=out)
    ctx.synchronize()
    for k in ("achtemp", "asxtemp", "acht_n1_loc"):
        np.testing.assert_array_equal(dev[k].cpu().numpy(), host[k])


def test_gpp_misaligned_device_arrays(ctx, fk):
    """Device arrays that start 8 bytes past a 16-byte boundary are copied into
    the workspace (the kernels move rows with 16-byte and bulk copies) and give
    the same bits as host arrays."""
    import ctypes
    import torch
    nb, nv, nc, ng = 70, 2, 1500, 11
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=13, dist="branch", wx="stress")
    keep = []

    def dev(a, dtype):
        raw = np.ascontiguousarray(a, dtype).view(np.uint8).ravel()
        t = torch.zeros(raw.size + 8, dtype=torch.uint8, device="cuda")
        t[8:] = torch.from_numpy(raw).cuda()
        keep.append(t)
        assert (t.data_ptr() + 8) % 16 == 8
        return ctypes.c_void_p(t.data_ptr() + 8)

    args = [dev(p["aqsmtemp"], np.complex128), dev(p["aqsntemp"], np.complex128),
            dev(p["I_eps_array"], np.complex128), dev(p["wtilde_array"], np.complex128),
            dev(p["vcoul"], np.float64), dev(p["inv_igp_index"], np.int32), dev(p["indinv"], np.int32),
            dev(p["wx_array"], np.float64)]
    for prec, code in (("fp64", fk.FK_FP64), ("mixed", fk.FK_MIXED)):
        want = ctx.gpp(p, prec)
        got = {"achtemp": np.zeros(3, np.complex128), "asxtemp": np.zeros(3, np.complex128),
               "acht_n1_loc": np.zeros(nb, np.complex128)}
        st = ctx.lib.fk_gpp(ctx.h, nb, nv, nc, ng, *args, code, 0,
                            *[ctypes.c_void_p(got[k].ctypes.data) for k in ("achtemp", "asxtemp", "acht_n1_loc")],
                            None)
        assert st == 0, ctx.lib.fk_last_error(ctx.h)
        for k in got:
            np.testing.assert_array_equal(got[k], want[k])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpp_bitwise_deterministic(ctx, fk, prec):
    p = fk.inputs.gpp_synthetic(200, 2, 3000, 24, seed=11, dist="uniform")
    a = ctx.gpp(p, prec)
    b = ctx.gpp(p, prec)
    for k in ("achtemp", "asxtemp", "acht_n1_loc"):
        np.testing.assert_array_equal(a[k], b[k])


def test_gpp_rejects_bad_arguments(ctx, fk):
    p = fk.inputs.gpp_synthetic(8, 2, 64, 4, seed=1)
    bad = dict(p, nvband=9)
    with pytest.raises(fk.FKError) as e:
        ctx.gpp(bad)
    assert e.value.status == 1
    q = fk.inputs.gpp_synthetic(8, 2, 16, 20, seed=1)  # ngpown > ncouls
    with pytest.raises(fk.FKError):
        ctx.gpp(q, "fp64", fk.FK_GPP_ROOT_QUIRKS)


def test_gpp_full_size_benchmark_config(ctx, fk, orc):
    """number_bands=512, nvband=2, ncouls=32768, ngpown=20 (the benchmark
    workload): FP64 against the oracle, mixed against FP64."""
    p = fk.inputs.gpp_synthetic(512, 2, 32768, 20, seed=2024, dist="uniform")
    # host bytes the call reads: all of aqsntemp, eps and wtilde, the small arrays, and only
    # the ngpown igp columns of aqsmtemp (gathered on the host)
    small = sum(np.asarray(p[k]).nbytes for k in ("vcoul", "inv_igp_index", "indinv", "wx_array"))
    expect = p["aqsntemp"].nbytes + p["I_eps_array"].nbytes + p["wtilde_array"].nbytes + 512 * 20 * 16 + small
    r64 = ctx.gpp(p, "fp64")
    assert ctx.last_transfer() == (expect, sum(v.nbytes for v in r64.values() if v is not None))
    check(r64, orc.gpp(p), TOL64)
    rmx = ctx.gpp(p, "mixed")  # large host arrays: the pipelined path (row blocks on a copy stream)
    assert ctx.last_transfer() == (expect, (7 + 512) * 16)  # outputs come back as one pinned block
    check(rmx, r64, TOLMX)   # plain relative error at the benchmark size


def test_gpp_full_size_reference_run(ctx, fk):
    """gppKer 512 2 32768 20 (ngpown = 1638), the reference's own canonical
    run, against the value its driver printed."""
    e = [x for x in golden("gppKer_bgw") if x["args"] == [512, 2, 32768, 20]]
    if not e:
        pytest.skip("full-size golden vector not generated")
    p = fk.inputs.gpp_reference_init(*e[0]["args"])
    driver_check(ctx.gpp(p, "fp64")["achtemp"], e[0], TOL64)
    driver_check(ctx.gpp(p, "mixed")["achtemp"], e[0], TOLMX)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpp_graph_replay_tracks_new_data(ctx, fk, prec):
    """Repeated device-resident calls are replayed from a captured CUDA graph;
    the replay must read the current contents of the (same) buffers."""
    import torch
    p = fk.inputs.gpp_synthetic(96, 2, 2000, 10, seed=12, dist="branch", wx="stress")
    d = dict(p)
    for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k])).cuda()
    for k in ("vcoul", "wx_array"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.float64)).cuda()
    for k in ("inv_igp_index", "indinv"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.int32)).cuda()
    out = {"achtemp": torch.zeros(3, dtype=torch.complex128, device="cuda"),
           "asxtemp": torch.zeros(3, dtype=torch.complex128, device="cuda"),
           "acht_n1_loc": torch.zeros(96, dtype=torch.complex128, device="cuda"), "achstemp": None}
    res = []
    for _ in range(4):  # eager, captured, replayed, replayed
        ctx.gpp(d, prec, out=out)
        ctx.synchronize()
        res.append(out["achtemp"].cpu().numpy().copy())
    for r in res[1:]:
        np.testing.assert_array_equal(r, res[0])
    d["aqsntemp"].mul_(2.0)  # every term is linear in aqsntemp; x2 is exact
    torch.cuda.synchronize()
    ctx.gpp(d, prec, out=out)
    ctx.synchronize()
    np.testing.assert_array_equal(out["achtemp"].cpu().numpy(), 2.0 * res[0])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_profiling_times_the_contraction_kernel(ctx, fk, prec):
    """With profiling on, the library brackets each launch of the dominant
    kernel with events: one launch for the plain sum, two for the half sum."""
    p = fk.inputs.gpp_synthetic(96, 2, 2000, 10, seed=15)
    ctx.set_profiling(True)
    try:
        ctx.gpp(p, prec)
        ms, n = ctx.last_kernel_time()
        assert n == 1 and 0 < ms < sum(ctx.last_timings())
        ctx.gpp(p, prec, fk.FK_GPP_HALF_SUM)
        ms2, n2 = ctx.last_kernel_time()
        assert n2 == 2 and ms2 > 0
    finally:
        ctx.set_profiling(False)


PHYS_CASES = [
    # (nb, nv, nc, ng, dist, index, wx)
    (512, 2, 2048, 64, "uniform", "even", "e10"),
    (64, 2, 777, 7, "branch", "reference", "stress"),
    (33, 5, 1000, 13, "branch", "even", "negative"),   # sexcut test of the Fortran source
    (40, 2, 2048, 16, "uniform", "even", "negative"),
]


@pytest.mark.parametrize("case", PHYS_CASES, ids=lambda c: "x".join(map(str, c[:4])) + "-" + c[6])
def test_gpp_physics_fp64_matches_oracle(ctx, fk, orc, case):
    """FK_GPP_PHYSICS (the Fortran source's ssx, sexcut test and asxtemp sign)
    against the oracle's physics mode; parity unpinned against the Fortran
    itself, which no compiler here can build."""
    nb, nv, nc, ng, dist, index, wx = case
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=nb + nc + 1, dist=dist, index=index, wx=wx)
    ref = orc.gpp(p, flags=orc.ORC_GPP_PHYSICS)
    check(ctx.gpp(p, "fp64", fk.FK_GPP_PHYSICS), ref, TOL64)


@pytest.mark.parametrize("case", PHYS_CASES, ids=lambda c: "x".join(map(str, c[:4])) + "-" + c[6])
def test_gpp_physics_mixed_within_1e6(ctx, fk, orc, case):
    nb, nv, nc, ng, dist, index, wx = case
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=nb + nc + 1, dist=dist, index=index, wx=wx)
    ref = ctx.gpp(p, "fp64", fk.FK_GPP_PHYSICS)
    check_mixed(ctx.gpp(p, "mixed", fk.FK_GPP_PHYSICS), ref, gpp_scales(p, orc, orc.ORC_GPP_PHYSICS))


def test_gpp_physics_rejects_other_drivers(ctx, fk):
    p = fk.inputs.gpp_synthetic(8, 2, 256, 4, seed=1)
    for extra in (fk.FK_GPP_ROOT_QUIRKS, fk.FK_GPP_HALF_SUM):
        with pytest.raises(fk.FKError) as e:
            ctx.gpp(p, "fp64", fk.FK_GPP_PHYSICS | extra)
        assert e.value.status == fk._native.FK_EINVAL
