"""The mixed path's a-priori error estimate (fk_set_error_estimate /
fk_gpp_error_estimate).

For every case the estimate of each output (achtemp and asxtemp: the largest
over the three frequencies; acht_n1_loc: the largest over the bands) must be
at least the measured error max |mixed - FP64| of that output, the FP64 path
standing in for exact arithmetic (its own error is ~1e-15 relative).  Where
the sums do not cancel (the benchmark-shaped uniform cases) the estimate must
also stay useful: at most 1e-4 of the output's magnitude.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("achtemp", "asxtemp", "acht_n1_loc")

CASES = [
    # (nb, nv, nc, ng, dist, index, wx, flags, useful)
    (512, 2, 2048, 64, "uniform", "even", "e10", 0, True),
    (64, 2, 777, 7, "branch", "reference", "stress", 0, False),
    (33, 5, 1000, 13, "branch", "even", "reference", 0, False),
    (16, 0, 640, 9, "uniform", "reference", "reference", 0, False),
    (12, 12, 300, 4, "branch", "reference", "stress", 0, False),
    (130, 2, 4099, 70, "branch", "reference", "stress", 0, False),
    (40, 3, 900, 9, "branch", "reference", "stress", "root", False),
    (33, 5, 1000, 13, "branch", "even", "negative", "physics", False),
    (512, 2, 8192, 16, "uniform", "even", "e10", 0, True),      # host arrays: pipelined path
    (512, 2, 32768, 20, "uniform", "even", "e10", 0, True),     # the benchmark workload
]


@pytest.fixture(scope="module")
def ectx(fk):
    c = fk.Context(0)
    c.set_error_estimate(True)
    yield c
    c.close()


def flag_of(fk, f):
    return {0: 0, "root": fk.FK_GPP_ROOT_QUIRKS, "physics": fk.FK_GPP_PHYSICS}[f]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:4])) + "-" + c[4] + "-" + str(c[7]))
def test_estimate_bounds_the_measured_error(ectx, fk, case):
    nb, nv, nc, ng, dist, index, wx, fl, useful = case
    p = fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=nb + nc + 3, dist=dist, index=index, wx=wx)
    flags = flag_of(fk, fl)
    ref = ectx.gpp(p, "fp64", flags)
    with pytest.raises(fk.FKError) as e:  # an FP64 call carries no estimate
        ectx.gpp_error_estimate()
    assert e.value.status == fk._native.FK_ENOTSUP
    res = ectx.gpp(p, "mixed", flags)
    est = ectx.gpp_error_estimate()
    for k in KEYS:
        err = float(np.max(np.abs(res[k] - ref[k])))
        mag = float(np.max(np.abs(ref[k])))
        print(f"estimate {k}: err {err:.3e} est {est[k]:.3e} ratio {err / est[k] if est[k] else 0:.3e} "
              f"est/|ref| {est[k] / mag if mag else 0:.3e}")
        assert np.isfinite(est[k]) and est[k] >= 0.0, (k, est[k])
        assert err <= est[k], (k, err, est[k])
        if useful and k != "asxtemp":
            assert est[k] <= 1e-4 * mag, (k, est[k], mag)


def test_estimate_follows_graph_replay(ectx, fk):
    # device-resident repeated calls replay a captured graph; the estimate is
    # recomputed by every replay
    import torch
    p = fk.inputs.gpp_synthetic(96, 2, 1024, 12, seed=5)
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
    ests = []
    for _ in range(4):  # eager, captured, replayed, replayed
        ectx.gpp(d, "mixed", 0, out=out)
        ests.append(ectx.gpp_error_estimate())
    assert ests[0] == ests[1] == ests[2] == ests[3]
    d["aqsntemp"].mul_(4.0)  # the same buffers: the replay recomputes the bound, which scales with |aqsntemp|
    torch.cuda.synchronize()
    ectx.gpp(d, "mixed", 0, out=out)
    e4 = ectx.gpp_error_estimate()
    for k in KEYS:
        assert e4[k] == pytest.approx(4.0 * ests[0][k], rel=1e-5), k


def test_estimate_off_and_half_sum_report_not_supported(fk):
    c = fk.Context(0)
    try:
        p = fk.inputs.gpp_synthetic(24, 2, 512, 6, seed=9)
        c.gpp(p, "mixed")
        with pytest.raises(fk.FKError) as e:  # estimate off
            c.gpp_error_estimate()
        assert e.value.status == fk._native.FK_ENOTSUP
        c.set_error_estimate(True)
        c.gpp(p, "mixed")
        assert all(v > 0 for v in c.gpp_error_estimate().values())
        c.gpp(p, "mixed", fk.FK_GPP_HALF_SUM)
        with pytest.raises(fk.FKError) as e:
            c.gpp_error_estimate()
        assert e.value.status == fk._native.FK_ENOTSUP
        c.set_error_estimate(False)
        c.gpp(p, "mixed")
        with pytest.raises(fk.FKError) as e:
            c.gpp_error_estimate()
        assert e.value.status == fk._native.FK_ENOTSUP
    finally:
        c.close()
