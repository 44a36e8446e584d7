"""Host-side failure handling on a GPU: allocations that cannot succeed
return FK_ENOMEM and leave the context usable, and a waiting served request
can be cancelled.  Nothing here faults, traps or hangs the GPU: the failures
are made on the host (an allocation larger than the device, a cancelled
ticket)."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def small(fk):
    return fk.inputs.gpp_synthetic(48, 2, 1536, 12, seed=1, dist="branch", index="reference", wx="reference")


def test_workspace_allocation_failure_leaves_context_usable(ctx, fk, orc):
    p = small(fk)
    before = ctx.gpp(p, "mixed")
    with pytest.raises(fk.FKError) as e:
        ctx.reserve(1 << 50)  # a petabyte: cudaMalloc must fail
    assert e.value.status == fk._native.FK_ENOMEM
    assert "cudaMalloc" in ctx.lib.fk_last_error(ctx.h).decode()
    for prec in ("fp64", "mixed"):
        r = ctx.gpp(p, prec)  # the workspace is allocated again on demand
        assert rel(r["achtemp"], orc.gpp(p)["achtemp"]) <= (1e-12 if prec == "fp64" else 1e-6)
    np.testing.assert_array_equal(ctx.gpp(p, "mixed")["achtemp"], before["achtemp"])


def test_server_memory_block_allocation_failure(fk):
    with pytest.raises(fk.FKError) as e:
        fk.Server(hbm_bytes=1 << 50, max_active=2)
    assert e.value.status == fk._native.FK_ENOMEM
    srv = fk.Server(hbm_bytes=256 << 20, max_active=2)  # the device is still usable
    try:
        out, _ = srv.wait(srv.submit(small(fk)))
        assert np.all(np.isfinite(out["achtemp"]))
    finally:
        srv.close()


def test_cancel_a_waiting_request(fk):
    """One active slot: while a long request runs, the next ones wait; one of
    them is cancelled (its outputs are never written), the running one cannot
    be, and the others complete."""
    import torch
    long_req = fk.inputs.gpp_synthetic(512, 2, 8192, 128, seed=3)
    d = dict(long_req)
    for k in ("aqsmtemp", "aqsntemp", "I_eps_array", "wtilde_array"):
        d[k] = torch.from_numpy(np.ascontiguousarray(long_req[k])).cuda()
    a, b = small(fk), fk.inputs.gpp_synthetic(64, 2, 2048, 16, seed=4)
    srv = fk.Server(hbm_bytes=2 << 30, max_active=1, step_stages=1)
    try:
        t_long = srv.submit(d)
        t_a = srv.submit(a, out={"achtemp": np.full(3, 7 + 7j), "asxtemp": np.full(3, 7 + 7j),
                                 "acht_n1_loc": np.full(a["number_bands"], 7 + 7j)})
        t_b = srv.submit(b)
        keep = srv._pending[t_a][1]
        assert srv.cancel(t_a) == fk._native.FK_OK
        assert srv.cancel(t_long) == fk._native.FK_EBUSY  # admitted: it runs to completion
        assert srv.cancel(987654321) == fk._native.FK_EINVAL
        with pytest.raises(fk.FKError) as e:
            srv.wait(t_a)
        assert e.value.status == fk._native.FK_ECANCELED
        assert np.all(keep["achtemp"] == 7 + 7j)  # never written
        out_long, _ = srv.wait(t_long)
        out_b, _ = srv.wait(t_b)
        info = srv.stats()
    finally:
        srv.close()
    assert info["completed"] >= 2
    assert np.all(np.isfinite(out_long["achtemp"])) and np.all(np.isfinite(out_b["achtemp"]))
