"""GPU tests of the bounded waits: a wait that gives up is reported as
FK_ETIMEOUT through the context's error word, the kernel returns normally
(its copies and MMAs in flight finish first), and the context stays usable.

No wait here is made to run out by breaking anything: the one-warp self-test
kernel waits on a barrier that nothing arrives on, and the contraction runs
with a wait bound of 0 cycles, so that any wait not satisfied on its first test
gives up."""
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def small_gpp(fk):
    return fk.inputs.gpp_synthetic(48, 2, 1536, 12, seed=1, dist="branch", index="reference", wx="reference")


def test_selftest_wait_times_out_and_context_recovers(ctx, fk, orc):
    for cycles in (0, 1000, 200000):
        assert ctx.selftest_timeout(cycles) == fk._native.FK_ETIMEOUT
        assert "self-test" in ctx.lib.fk_last_error(ctx.h).decode()
    p = small_gpp(fk)
    ref = orc.gpp(p)
    r = ctx.gpp(p, "mixed")  # the error word was cleared: a normal call succeeds
    assert rel(r["achtemp"], ref["achtemp"]) <= 1e-6


@pytest.mark.parametrize("path", ["gpp", "ff"])
def test_contraction_wait_timeout_is_reported(ctx, fk, orc, path):
    if path == "gpp":
        p = small_gpp(fk)
        call = lambda: ctx.gpp(p, "mixed")
        ref = orc.gpp(p)
        keys = ("achtemp", "asxtemp")
    else:
        p = fk.inputs.ff_synthetic(40, 2, 640, 48, 6, 5, seed=2)
        call = lambda: ctx.ff(p, "mixed", fk.FK_FF_SCHDT_GEMM)
        ref = orc.ff(p, flags=orc.ORC_FF_SCHDT_GEMM)
        keys = ("achsDtemp", "schDt_matrix")
    ctx.set_wait_limit(0)
    try:
        for _ in range(2):
            with pytest.raises(fk.FKError) as e:
                call()
            assert e.value.status == fk._native.FK_ETIMEOUT
            assert "timed out" in str(e.value)
    finally:
        ctx.set_wait_limit(-1)
    ctx.synchronize()
    r = call()  # default bound again: the same context gives the right result
    for k in keys:
        assert rel(r[k], ref[k]) <= 1e-5, k
