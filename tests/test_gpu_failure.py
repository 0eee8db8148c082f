"""Failure detection without a GPU fault: the windowed back-projection's
pipeline waits are bounded, and a test makes them give up.

mtr_set_wait_limit(0) makes every producer / consumer wait of the kernel give
up at once: the launch flags itself, drains its own TMA copies (with the full
bound) and returns, so nothing hangs and no copy is left in flight.  The
host then reads MTR_ERR_TIMEOUT from mtr_recon_check, and the same context
reconstructs correctly once the default bound is restored."""
import pytest

import cases
import mtr
import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_waits_that_give_up_report_timeout_and_the_context_recovers(ctx):
    c = cases.get("mid_oblique")
    p = mtr.params(iter_times=1, sirt_inner=2, sirt_step=0.5, mace_step=0.7)
    r = mtr.Recon(ctx, c.axes, c.vol, p)  # tiles tuned with the default bound
    lib = ctx.lib
    n0 = ctx.windowed_launch_count()
    assert lib.mtr_set_wait_limit(0) == mtr.OK
    try:
        r.run()
        st = lib.mtr_recon_check(r.h)
    finally:
        lib.mtr_set_wait_limit(-1)
    assert ctx.windowed_launch_count() > n0  # the windowed back-projection ran
    assert st == mtr.ERR_TIMEOUT
    assert b"bounded wait" in lib.mtr_context_last_error(ctx.h)
    r.close()
    # the same context, default bound: a reconstruction gives the oracle's result
    got = ctx.reconstruct(c.axes, c.vol, p)
    want = oracle.reconstruct(oracle.REF_FAITHFUL, c.axes, c.vol, 1, 2, 0.5, 0.7)
    assert rel_l2(got, want) < 1e-4
