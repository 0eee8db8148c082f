"""Reconstruction arrays from the context's stream-ordered pool: arrays that
come back from the pool hold the previous reconstruction's data, and a
reconstruction on reused arrays (of another size in between) equals one on
a fresh context within the bound two identical runs keep."""
import numpy as np
import pytest

import cases
import mtr
from conftest import rel_l2, run_to_run_tol

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [mtr.PREC_FP32, mtr.PREC_MIXED_BF16])
def test_reused_arrays_give_the_same_result(prec):
    a, b = cases.get("two_axis"), cases.get("mid")
    p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec)
    with mtr.Context(0) as fresh:
        want_a = fresh.reconstruct(a.axes, a.vol, p)
    with mtr.Context(0) as fresh:
        want_b = fresh.reconstruct(b.axes, b.vol, p)
    with mtr.Context(0) as ctx:
        got = []
        for c in (a, b, a, b, a):
            got.append(ctx.reconstruct(c.axes, c.vol, p))
        tol = run_to_run_tol(prec)
        for i, g in enumerate(got):
            want = want_a if i % 2 == 0 else want_b
            assert np.isfinite(g).all()
            assert rel_l2(g, want) < tol, i
        # the reserve can be returned at any time; later runs allocate anew
        ctx.trim()
        assert rel_l2(ctx.reconstruct(a.axes, a.vol, p), want_a) < tol
