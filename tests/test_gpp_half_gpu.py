"""GPU parity tests of the half-sum GPP mode (FK_GPP_HALF_SUM, gppsum == 1 of
gppKerSeq.cpp) through the C ABI against the oracle.

For column igp the sum runs over ig below igp, in the reference program's 512-wide
blocks (which skip ig = 511 mod 512 and add the diagonal ig = igp when igp is
a multiple of 512), and each term carries its conjugate pair.  The cases put
columns on both sides of those block edges.

Tolerances (relative, normwise over each output vector):
  FP64 path  <= 1e-12 against the oracle;
  mixed path <= 1e-6 against the FP64 path (scaled by the rss of the terms).
"""
import json
import os

import numpy as np
import pytest

from conftest import gpp_scales, mixed_gate, rel

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64, TOLMX = 1e-12, 1e-6
KEYS = ("achtemp", "asxtemp", "acht_n1_loc")

# columns on and around the 512-wide block edges, the first columns and the last
EDGE_COLS = [0, 1, 2, 510, 511, 512, 513, 1023, 1024, 1025, 1535, 1536, 1537]


def half_inputs(fk, nb, nv, nc, ng, seed, dist, wx):
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=seed, dist=dist, index="even", wx=wx)
    cols = [c for c in EDGE_COLS if c < nc] + [nc - 2, nc - 1, nc // 3]
    rng = np.random.default_rng(seed)
    extra = rng.integers(0, nc, size=max(0, ng - len(cols)))
    p["inv_igp_index"] = np.ascontiguousarray((cols + list(extra))[:ng], np.int32)
    p["indinv"] = np.arange(nc, dtype=np.int32)
    return p


CASES = [
    # (nb, nv, nc, ng, dist, wx)
    (64, 2, 2048, 19, "branch", "stress"),      # every block edge up to 1537, every branch
    (40, 5, 1600, 16, "uniform", "e10"),   # three flag passes
    (12, 12, 1100, 9, "branch", "reference"),   # all bands occupied
    (16, 0, 1030, 9, "branch", "stress"),       # no occupied bands
    (130, 2, 4099, 70, "uniform", "stress"),    # ragged tiles
    (1, 1, 64, 3, "branch", "stress"),          # smallest
]


def ids(c):
    return "x".join(map(str, c[:4])) + "-" + c[4]


@pytest.mark.parametrize("case", CASES, ids=ids)
def test_half_sum_fp64_matches_oracle(ctx, fk, orc, case):
    nb, nv, nc, ng, dist, wx = case
    p = half_inputs(fk, nb, nv, nc, ng, nb + nc, dist, wx)
    ref = orc.gpp(p, flags=orc.ORC_GPP_HALF_SUM)
    res = ctx.gpp(p, "fp64", fk.FK_GPP_HALF_SUM)
    errs = {k: rel(res[k], ref[k]) for k in KEYS if np.max(np.abs(ref[k])) > 0}
    assert all(e <= TOL64 for e in errs.values()), errs


@pytest.mark.parametrize("case", CASES, ids=ids)
def test_half_sum_mixed_within_1e6(ctx, fk, orc, case):
    nb, nv, nc, ng, dist, wx = case
    p = half_inputs(fk, nb, nv, nc, ng, nb + nc, dist, wx)
    ref = ctx.gpp(p, "fp64", fk.FK_GPP_HALF_SUM)
    res = ctx.gpp(p, "mixed", fk.FK_GPP_HALF_SUM)
    scales = gpp_scales(p, orc, orc.ORC_GPP_HALF_SUM)
    mixed_gate(res, ref, scales, TOLMX)


def seq_entries():
    with open(os.path.join(GOLD, "reference_drivers.json")) as f:
        return json.load(f)["gppKer_seq"]


@pytest.mark.parametrize("entry", seq_entries(), ids=lambda e: "x".join(map(str, e["args"])))
def test_half_sum_matches_seq_driver_prints(ctx, fk, entry):
    """gppKerSeq.cpp with gppsum = 1 on its own constant inputs: the printed
    achtemp (the oracle matches it to 1e-13)."""
    nb, nv, nc, npg, gppsum = entry["args"]
    assert gppsum == 1
    p = fk.inputs.gpp_reference_init(nb, nv, nc, npg)
    printed = np.array([complex(*z) for z in entry["achtemp"]])
    assert rel(ctx.gpp(p, "fp64", fk.FK_GPP_HALF_SUM)["achtemp"], printed) <= TOL64
    assert rel(ctx.gpp(p, "mixed", fk.FK_GPP_HALF_SUM)["achtemp"], printed) <= TOLMX


def test_half_sum_benchmark_size(ctx, fk, orc):
    """512 x 2 x 32768 x 20: FP64 against the oracle, mixed against FP64."""
    p = fk.inputs.gpp_synthetic(512, 2, 32768, 20, seed=77, dist="uniform")
    r64 = ctx.gpp(p, "fp64", fk.FK_GPP_HALF_SUM)
    ref = orc.gpp(p, flags=orc.ORC_GPP_HALF_SUM)
    for k in KEYS:
        assert rel(r64[k], ref[k]) <= TOL64, k
    rmx = ctx.gpp(p, "mixed", fk.FK_GPP_HALF_SUM)
    for k in ("achtemp", "acht_n1_loc"):
        assert rel(rmx[k], r64[k]) <= TOLMX, k


def test_half_sum_device_arrays_equal_host_arrays(ctx, fk):
    import torch
    nb = 70
    p = half_inputs(fk, nb, 3, 1500, 11, 14, "branch", "stress")
    for prec in ("fp64", "mixed"):
        host = ctx.gpp(p, prec, fk.FK_GPP_HALF_SUM)
        d = dict(p)
        for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array"):
            d[k] = torch.from_numpy(np.ascontiguousarray(p[k])).cuda()
        for k in ("vcoul", "wx_array"):
            d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.float64)).cuda()
        for k in ("inv_igp_index", "indinv"):
            d[k] = torch.from_numpy(np.ascontiguousarray(p[k], np.int32)).cuda()
        out = {k: torch.zeros(n, dtype=torch.complex128, device="cuda")
               for k, n in (("achtemp", 3), ("asxtemp", 3), ("acht_n1_loc", nb))}
        out["achstemp"] = None
        for _ in range(3):  # eager, then captured and replayed
            ctx.gpp(d, prec, fk.FK_GPP_HALF_SUM, out=out)
            ctx.synchronize()
            for k in KEYS:
                np.testing.assert_array_equal(out[k].cpu().numpy(), host[k])


def test_half_sum_rejects_other_drivers(ctx, fk):
    p = fk.inputs.gpp_synthetic(8, 2, 64, 4, seed=1)
    with pytest.raises(fk.FKError) as e:
        ctx.gpp(p, "fp64", fk.FK_GPP_HALF_SUM | fk.FK_GPP_ROOT_QUIRKS)
    assert e.value.status == 1
    with pytest.raises(fk.FKError) as e:
        ctx.gpp(p, "fp64", fk.FK_GPP_HALF_SUM | fk.FK_GPP_ACHSTEMP)
    assert e.value.status == 6
