"""Serving (mtr_server_*): continuous batching with admission by device
footprint.  A request's result must not depend on the mix it was served
in, must equal the same reconstruction run alone through mtr_reconstruct,
and admission must keep the admitted footprint within the budget."""
import numpy as np
import pytest

import cases
import mtr
from conftest import rel_l2, run_to_run_tol

pytestmark = pytest.mark.gpu

MIX = ["mid_oblique", "two_axis", "four_axis", "single", "oob"]


def _serve(ctx, reqs, budget=1 << 40, precision=mtr.PREC_FP32, arrive=None):
    """reqs: [(case, iter_times, sirt_inner)]; arrive[i] = step at which request i is submitted."""
    srv = mtr.Server(ctx, budget, precision)
    arrive = arrive or [0] * len(reqs)
    ids, done, step = {}, {}, 0
    while len(done) < len(reqs):
        for i, (c, no, ni) in enumerate(reqs):
            if arrive[i] == step:
                ids[srv.submit(c.axes, c.vol, no, ni, 0.5, 0.8)] = i
        for rid, vol in srv.step():
            done[ids[rid]] = vol
        step += 1
        assert step < 10000
    st = srv.stats()
    srv.close()
    return [done[i] for i in range(len(reqs))], st


@pytest.mark.parametrize("prec", [mtr.PREC_FP32, mtr.PREC_MIXED_BF16])
def test_alone_equals_in_mix(ctx, prec):
    target = (cases.get("mid"), 2, 3)
    alone, _ = _serve(ctx, [target], precision=prec)
    mix = [target] + [(cases.get(n), 1 + i % 2, 2 + i) for i, n in enumerate(MIX)]
    arrive = [2, 0, 1, 3, 3, 5]
    got, st = _serve(ctx, mix, precision=prec, arrive=arrive)
    assert st["completed"] == len(mix)
    tol = run_to_run_tol(prec)
    assert rel_l2(got[0], alone[0]) < tol
    # and the mix members equal their own single-request runs
    want = ctx.reconstruct(target[0].axes, target[0].vol,
                           mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec))
    assert rel_l2(got[0], want) < tol
    for (c, no, ni), v in zip(mix[1:], got[1:]):
        ref = ctx.reconstruct(c.axes, c.vol, mtr.params(iter_times=no, sirt_inner=ni, sirt_step=0.5, mace_step=0.8,
                                                         precision=prec))
        assert rel_l2(v, ref) < tol


def test_mixed_vs_fp32_served(ctx):
    reqs = [(cases.get(n), 2, 3) for n in ("mid", "mid_oblique", "two_axis")]
    f32, _ = _serve(ctx, reqs, precision=mtr.PREC_FP32)
    bf, _ = _serve(ctx, reqs, precision=mtr.PREC_MIXED_BF16)
    for a, b in zip(f32, bf):
        assert rel_l2(b, a) < 1e-3


def test_admission_respects_budget(ctx):
    cs = [cases.get(n) for n in ("mid", "mid_oblique", "two_axis")]
    fps = [mtr.estimate_footprint([(a.prj.X, a.prj.Y, a.prj.AngN) for a in c.axes], c.vol, mtr.PREC_FP32) for c in cs]
    budget = max(fps) + min(fps) // 2  # never two of the larger ones at once
    got, st = _serve(ctx, [(c, 1, 2) for c in cs], budget=budget)
    assert st["completed"] == 3 and st["peak_bytes"] <= budget
    for c, v in zip(cs, got):
        ref = ctx.reconstruct(c.axes, c.vol, mtr.params(iter_times=1, sirt_inner=2, sirt_step=0.5, mace_step=0.8))
        assert rel_l2(v, ref) < 1e-5


def test_request_over_budget_is_refused(ctx):
    c = cases.get("mid")
    srv = mtr.Server(ctx, 1 << 20)
    with pytest.raises(mtr.MtrError) as e:
        srv.submit(c.axes, c.vol, 1, 1)
    assert e.value.status == mtr.ERR_CAPACITY
    srv.close()


def test_zero_iterations_returns_wbp_sum(ctx):
    c = cases.get("two_axis")
    got, _ = _serve(ctx, [(c, 0, 10)])
    ref = ctx.reconstruct(c.axes, c.vol, mtr.params(iter_times=0, sirt_inner=10))
    np.testing.assert_allclose(got[0], ref, rtol=1e-6, atol=1e-6)
