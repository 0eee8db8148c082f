"""Batched reconstruction (one persistent launch per SIRT phase over many
instances, CUDA graph): every instance's result must match the same
instance reconstructed alone, and graph replays must repeat it."""
import numpy as np
import pytest

import cases
import mtr
import oracle
from conftest import rel_l2, run_to_run_tol

pytestmark = pytest.mark.gpu

NAMES = ["mid", "mid_oblique", "two_axis", "four_axis", "single"]


# Tiles pinned so that the persistent kernels (warp lines) and the own
# launches of patch-tiled axes are both exercised; None = tuned.
@pytest.mark.parametrize("tiles", ["8,16,0,0", "16,16,2,2", None])
@pytest.mark.parametrize("prec", [mtr.PREC_FP32, mtr.PREC_MIXED_BF16])
def test_batch_matches_each_instance_alone(ctx, monkeypatch, prec, tiles):
    if tiles:
        monkeypatch.setenv("MTR_FORCE_DEPTHS", tiles)
    cs = [cases.get(n) for n in NAMES]
    p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec, flags=mtr.FLAG_GRAPH)
    b = mtr.Batch(ctx, [(c.axes, c.vol) for c in cs], p)
    info = b.info()
    if tiles == "8,16,0,0":
        assert info["items"]["forward"] > 0 and info["items"]["backproject"] > 0
    if tiles == "16,16,2,2":
        assert info["items"]["own_launch_axes"] > 0
    b.run()
    first = [b.download(i) for i in range(len(cs))]
    b.run()  # graph replay
    second = [b.download(i) for i in range(len(cs))]
    b.close()
    alone_p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec)
    for c, got, again in zip(cs, first, second):
        alone = ctx.reconstruct(c.axes, c.vol, alone_p)
        assert rel_l2(got, alone) < run_to_run_tol(prec)
        assert rel_l2(again, got) < run_to_run_tol(prec)


def test_batch_matches_oracle(ctx):
    cs = [cases.get(n) for n in ("mid", "two_axis")]
    p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, flags=mtr.FLAG_GRAPH)
    b = mtr.Batch(ctx, [(c.axes, c.vol) for c in cs], p)
    b.run()
    for i, c in enumerate(cs):
        want = oracle.reconstruct(oracle.REF_FAITHFUL, c.axes, c.vol, 2, 3, 0.5, 0.8)
        assert rel_l2(b.download(i), want) < 1e-4
    b.close()


def test_batch_without_graph(ctx):
    c = cases.get("mid_oblique")
    p = mtr.params(iter_times=1, sirt_inner=2, sirt_step=0.5, mace_step=0.7)
    b = mtr.Batch(ctx, [(c.axes, c.vol), (c.axes, c.vol)], p)
    b.run()
    a0, a1 = b.download(0), b.download(1)
    b.close()
    np.testing.assert_allclose(a0, a1, rtol=1e-6, atol=1e-6)
