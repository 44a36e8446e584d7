"""The GPP request server (fk_server_*): served results against fk_gpp, the
same result alone and in a mix, resident epsilon/wtilde, memory-gated
admission.

Tolerances: a served request runs the mixed path, so its outputs are within
1e-6 (relative, normwise) of fk_gpp's FP64 path; alone and in a mix the same
request gives bit-identical outputs (its k-slices and summation order depend
only on its own shape).
"""
import numpy as np
import pytest

from conftest import gpp_scales_torch, mixed_gate, rel

pytestmark = pytest.mark.gpu
TOL = 1e-6
KEYS = ("achtemp", "asxtemp", "acht_n1_loc")

# (nb, nv, nc, ng, dist, wx): uneven sizes, every branch, a request with no
# contraction units (all bands occupied)
REQS = [
    (256, 2, 4096, 64, "uniform", "e10"),
    (128, 2, 2048, 32, "branch", "stress"),
    (512, 2, 8192, 128, "uniform", "e10"),
    (96, 5, 3000, 47, "branch", "reference"),
    (12, 12, 300, 4, "branch", "stress"),
    (1024, 2, 2048, 32, "uniform", "e10"),
]


def make(fk, i, c):
    nb, nv, nc, ng, dist, wx = c
    return fk.inputs.gpp_synthetic(nb, nv, nc, ng, seed=100 + i, dist=dist, wx=wx)


@pytest.fixture(scope="module")
def reqs(fk):
    return [make(fk, i, c) for i, c in enumerate(REQS)]


@pytest.fixture(scope="module")
def ref64(ctx, reqs):
    return [ctx.gpp(p, "fp64") for p in reqs]


def test_served_requests_match_fk_gpp(fk, reqs, ref64):
    srv = fk.Server(hbm_bytes=4 << 30, max_active=8)
    try:
        for p, want in zip(reqs, ref64):
            out, lat = srv.wait(srv.submit(p))
            assert lat > 0
            for k in KEYS:
                assert rel(out[k], want[k]) <= TOL, k
    finally:
        srv.close()


def test_same_result_alone_and_in_the_mix(fk, reqs):
    # alone: one request at a time; mix: all at once, with a small step so
    # that large requests span several steps interleaved with the others
    alone = []
    srv = fk.Server(hbm_bytes=4 << 30, max_active=8, step_stages=8)
    try:
        for p in reqs:
            alone.append(srv.wait(srv.submit(p))[0])
        tickets = [srv.submit(p) for p in reqs]
        mixed = [srv.wait(t)[0] for t in tickets]
        info = srv.stats()
    finally:
        srv.close()
    assert info["mean_active"] > 1.0 and info["steps"] > len(reqs)
    for a, b in zip(alone, mixed):
        for k in KEYS:
            np.testing.assert_array_equal(a[k], b[k])


def test_resident_epsilon_and_wtilde(fk, reqs):
    import torch
    p = reqs[0]
    srv = fk.Server(hbm_bytes=2 << 30, max_active=4)
    try:
        direct = srv.wait(srv.submit(p))[0]
        srv.resident_put(7, p["I_eps_array"])
        srv.resident_put(8, torch.from_numpy(np.ascontiguousarray(p["wtilde_array"])).cuda())
        outs = [srv.wait(t)[0] for t in [srv.submit(p, eps_key=7, wtilde_key=8) for _ in range(3)]]
        srv.resident_evict(7)
        srv.resident_evict(8)
        with pytest.raises(fk.FKError):
            srv.submit(p, eps_key=7, wtilde_key=8)
    finally:
        srv.close()
    for o in outs:
        for k in KEYS:
            np.testing.assert_array_equal(o[k], direct[k])


def test_admission_is_gated_by_memory(fk, reqs, ref64):
    import torch
    # device-resident inputs; a budget that holds about two of these requests' workspaces
    p = reqs[2]
    d = dict(p)
    for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array"):
        d[k] = torch.from_numpy(np.ascontiguousarray(p[k])).cuda()
    budget = 100 << 20
    srv = fk.Server(hbm_bytes=budget, max_active=16, step_stages=16)
    try:
        tickets = [srv.submit(d) for _ in range(6)]
        outs = [srv.wait(t)[0] for t in tickets]
        info = srv.stats()
        big = make(fk, 9, (16, 2, 32768, 128, "uniform", "e10"))  # its image alone is ~150 MB
        with pytest.raises(fk.FKError) as e:
            srv.submit(big)
        assert e.value.status == fk._native.FK_ENOMEM
    finally:
        srv.close()
    assert info["completed"] == 6 and info["hbm_peak_bytes"] <= budget
    assert info["peak_active"] < 6
    for o in outs:
        for k in KEYS:
            assert rel(o[k], ref64[2][k]) <= TOL, k


def test_autotuned_plan(fk, reqs, ref64):
    """The tuner picks a k-split for a shape; requests of that shape then use
    it and stay within tolerance, alone and in a mix."""
    p = reqs[2]
    srv = fk.Server(hbm_bytes=4 << 30, max_active=8, step_stages=8)
    try:
        with pytest.raises(fk.FKError):
            srv.tune(p["number_bands"], p["nvband"], p["ncouls"], 0)
        ks = srv.tune(p["number_bands"], p["nvband"], p["ncouls"], p["ngpown"])
        assert ks >= 1
        alone = srv.wait(srv.submit(p))[0]
        tickets = [srv.submit(q) for q in reqs]
        mixed = [srv.wait(t)[0] for t in tickets]
    finally:
        srv.close()
    for k in KEYS:
        assert rel(alone[k], ref64[2][k]) <= TOL, k
        np.testing.assert_array_equal(mixed[2][k], alone[k])


def test_served_uneven_stream_request_shapes(fk, ctx):
    """The served stream's request shapes at their real sizes: every
    number_bands value of the stream (128, 256, 512, 1024) at both ends of
    its ncouls range (2048 and 32768), ngpown = ncouls / 64, nvband 2, the
    benchmark distributions, epsilon and wtilde resident.  Each result is
    within plain relative error 1e-6 of fk_gpp's FP64 path, and the same bits
    alone and in the mix."""
    import torch
    shapes = [(nb, nc) for nc in (2048, 32768) for nb in (128, 256, 512, 1024)]
    pools = {nc: fk.inputs.gpp_synthetic(1024, 2, nc, nc // 64, seed=nc) for nc in (2048, 32768)}
    dev = {nc: {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() if isinstance(v, np.ndarray) else v
                for k, v in q.items()} for nc, q in pools.items()}

    def request(nb, nc):
        q = dict(dev[nc])
        q["number_bands"] = nb
        q["aqsmtemp"], q["aqsntemp"] = q["aqsmtemp"][:nb], q["aqsntemp"][:nb]
        return q

    want = {s: ctx.gpp(request(*s), "fp64") for s in shapes}  # host outputs: the call waits for its stream
    srv = fk.Server(hbm_bytes=12 << 30, max_active=16, step_stages=32)
    try:
        for i, nc in enumerate((2048, 32768)):
            srv.resident_put(10 + 2 * i, dev[nc]["I_eps_array"])
            srv.resident_put(11 + 2 * i, dev[nc]["wtilde_array"])
        keys = {2048: (10, 11), 32768: (12, 13)}

        def submit(nb, nc):
            return srv.submit(request(nb, nc), eps_key=keys[nc][0], wtilde_key=keys[nc][1])

        alone = {s: srv.wait(submit(*s))[0] for s in shapes}
        tickets = {s: submit(*s) for s in shapes}
        mixed = {s: srv.wait(t)[0] for s, t in tickets.items()}
        info = srv.stats()
    finally:
        srv.close()
    assert info["mean_active"] > 1.0
    for s in shapes:
        # plain relative error, except for outputs that cancel (see mixed_gate)
        mixed_gate(alone[s], want[s], gpp_scales_torch(request(*s)), TOL, keys=KEYS)
        for k in KEYS:
            np.testing.assert_array_equal(mixed[s][k], alone[s][k])
