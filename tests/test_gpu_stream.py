"""The single-GPU streaming slab loop (MTR_FLAG_STREAM_SLABS) against the
unsplit, device-resident run of the same reconstruction.

The streamed run keeps every volume-sized array in host memory and moves
Z-slabs through a two-slot device working set; its ray sums are the sum of
the slabs' splats, as the reference reduces its Z-slab ranks' partial sums
(FunctionOnGPU.cu:218-238).  Slab depths below cover a ragged last slab,
depths that are not a multiple of the kernels' brick depth, one-plane slabs,
the windowed and the plain kernels, one to four axes and both precisions."""
import numpy as np
import pytest

import cases
import mtr
import oracle
from conftest import rel_l2, run_to_run_tol

pytestmark = pytest.mark.gpu


def _run(ctx, c, p):
    r = mtr.Recon(ctx, c.axes, c.vol, p)
    r.run()
    out = r.download()
    fp = r.footprint()
    r.close()
    return out, fp


@pytest.mark.parametrize("name,depth,prec", [("mid", 8, mtr.PREC_FP32), ("mid", 3, mtr.PREC_FP32),
                                             ("mid_oblique", 7, mtr.PREC_FP32), ("mid_oblique", 7, mtr.PREC_MIXED_BF16),
                                             ("four_axis", 2, mtr.PREC_FP32), ("single", 1, mtr.PREC_FP32),
                                             ("mid", 32, mtr.PREC_MIXED_FP16)])
def test_streamed_slabs_equal_the_unsplit_run(ctx, name, depth, prec):
    c = cases.get(name)
    kw = dict(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec)
    want, fp_dev = _run(ctx, c, mtr.params(**kw))
    got, fp_str = _run(ctx, c, mtr.params(**kw, flags=mtr.FLAG_STREAM_SLABS, slab_depth=depth))
    assert rel_l2(got, want) < run_to_run_tol(prec)
    if depth < c.vol.Z:  # several slabs: the working set is smaller than the volume arrays
        assert fp_str < fp_dev


def test_streamed_slabs_match_the_oracle_and_record_norms(ctx):
    c = cases.get("mid_oblique")
    p = mtr.params(iter_times=1, sirt_inner=4, sirt_step=0.5, mace_step=0.7,
                   flags=mtr.FLAG_STREAM_SLABS | mtr.FLAG_RECORD_NORMS | mtr.FLAG_RECORD_CHANGES, slab_depth=5)
    r = mtr.Recon(ctx, c.axes, c.vol, p)
    r.run()
    got = r.download()
    norms = r.norms()
    assert r.changes(1)[0] > 0
    r.close()
    want, want_n = oracle.reconstruct(oracle.REF_FAITHFUL, c.axes, c.vol, 1, 4, 0.5, 0.7, with_norms=True)
    assert rel_l2(got, want) < 1e-4
    np.testing.assert_allclose(norms, want_n, rtol=1e-4)


def test_streamed_run_in_pieces_and_resumed(ctx, tmp_path):
    """init + run_outer in pieces, checkpoint and resume: the same state as a
    run in one go (the volume arrays it saves and restores are host arrays)."""
    c = cases.get("two_axis")
    p = mtr.params(iter_times=3, sirt_inner=2, sirt_step=0.5, mace_step=0.8, flags=mtr.FLAG_STREAM_SLABS,
                   slab_depth=4)
    whole, _ = _run(ctx, c, p)
    r = mtr.Recon(ctx, c.axes, c.vol, p)
    r.init()
    r.run_outer(0, 1)
    r.save(tmp_path / "ck.bin")
    r.close()
    r2 = mtr.Recon(ctx, c.axes, c.vol, p)
    done = r2.load(tmp_path / "ck.bin")
    assert done == 1
    r2.run_outer(1, 2)
    got = r2.download()
    r2.close()
    assert rel_l2(got, whole) < 1e-5
