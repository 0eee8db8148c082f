"""GPU parity: libmtr (through its C ABI) against the CPU oracle and, where
the prebuilt cubin is present, against the reference's own CUDA kernels.

Bounds (relative L2 per volume):
  FP32 path vs reference-faithful oracle / reference kernels: 1e-4
  mixed precision vs the FP64 oracle:                          1e-3
"""
import numpy as np
import pytest

import cases
import mtr
import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4
MIXED_TOL = 1e-3


@pytest.mark.parametrize("name", ["single", "two_axis", "oob", "four_axis", "rect"])
def test_wbp_matches_oracle(ctx, name):
    c = cases.get(name)
    for a in c.axes:
        got = ctx.wbp(a, c.vol)
        want = oracle.wbp(oracle.REF_FAITHFUL, a, c.vol)
        assert rel_l2(got, want) < 1e-5


def test_wbp_slab_matches_full_volume(ctx):
    c = cases.get("single")
    v = c.vol
    full = ctx.wbp(c.axes[0], v)
    lo = ctx.wbp(c.axes[0], v, v.Zstart, v.Zstart + 3)
    hi = ctx.wbp(c.axes[0], v, v.Zstart + 3, v.Zend)
    # Not bit-identical: each CTA evaluates the map in FP64 at its own base
    # voxel, and the slab origin moves that base.
    assert rel_l2(np.concatenate([lo, hi]), full) < 1e-6


@pytest.mark.parametrize("name", ["single", "oob", "rect"])
def test_sirt_matches_oracle(ctx, name):
    c = cases.get(name)
    a = c.axes[0]
    x0 = oracle.wbp(oracle.REF_FAITHFUL, a, c.vol).astype(np.float32)
    got = ctx.sirt(a, c.vol, x0, n_inner=6, step=0.5)
    want = oracle.sirt(oracle.REF_FAITHFUL, a, c.vol, x0, 6, 0.5)
    assert rel_l2(got, want) < FP32_TOL


@pytest.mark.parametrize("name,no,ni,rho", [("single", 1, 10, 0.5), ("two_axis", 2, 3, 0.8),
                                            ("four_axis", 2, 2, 0.7), ("oob", 1, 3, 0.7)])
def test_reconstruct_matches_oracle(ctx, name, no, ni, rho):
    c = cases.get(name)
    p = mtr.params(iter_times=no, sirt_inner=ni, sirt_step=0.5, mace_step=rho)
    got = ctx.reconstruct(c.axes, c.vol, p)
    want = oracle.reconstruct(oracle.REF_FAITHFUL, c.axes, c.vol, no, ni, 0.5, rho)
    assert rel_l2(got, want) < FP32_TOL


@pytest.mark.parametrize("prec", [mtr.PREC_MIXED_BF16, mtr.PREC_MIXED_FP16])
def test_mixed_precision_vs_fp64(ctx, prec):
    c = cases.get("two_axis")
    p = mtr.params(iter_times=2, sirt_inner=4, sirt_step=0.5, mace_step=0.8, precision=prec)
    got = ctx.reconstruct(c.axes, c.vol, p)
    want = oracle.reconstruct(oracle.FP64, c.axes, c.vol, 2, 4, 0.5, 0.8)
    assert rel_l2(got, want) < MIXED_TOL


def test_graph_replay_matches_direct(ctx):
    c = cases.get("two_axis")
    p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8)
    direct = ctx.reconstruct(c.axes, c.vol, p)
    pg = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, flags=mtr.FLAG_GRAPH)
    r = mtr.Recon(ctx, c.axes, c.vol, pg)
    r.run()
    first = r.download()
    r.run()  # replay
    second = r.download()
    # per-kernel profiling runs the launches one by one, between their events
    ctx.profile_reset()
    ctx.set_profiling(True)
    try:
        r.run()
        third = r.download()
    finally:
        ctx.set_profiling(False)
    prof = ctx.profile()
    r.close()
    assert rel_l2(first, direct) < 1e-5
    assert rel_l2(second, first) < 1e-5
    assert rel_l2(third, first) < 1e-5
    assert prof["forward"][0] == 2 * 2 * 3 and prof["backproject"][0] > 0


def test_residual_norms_decrease_and_match_oracle(ctx):
    c = cases.get("single")
    p = mtr.params(iter_times=1, sirt_inner=8, sirt_step=0.5, mace_step=0.5, flags=mtr.FLAG_RECORD_NORMS)
    r = mtr.Recon(ctx, c.axes, c.vol, p)
    r.run()
    n = r.norms()[0, 0]
    r.close()
    _, want = oracle.reconstruct(oracle.FP64, c.axes, c.vol, 1, 8, 0.5, 0.5, with_norms=True)
    assert np.all(np.diff(n) < 0)
    np.testing.assert_allclose(n, want[0, 0], rtol=1e-4)


def test_elementwise_bit_exact(ctx):
    rng = np.random.default_rng(5)
    v = mtr.VolumeSize.make(0, 17, 0, 9, 0, 3)
    w = rng.normal(size=v.shape).astype(np.float32)
    wa = rng.normal(size=v.shape).astype(np.float32)
    z = ctx.initial_z(v, w, wa)
    np.testing.assert_array_equal(z, (np.float32(2) * wa - w).astype(np.float32))
    vv = rng.normal(size=v.shape).astype(np.float32)
    step = np.float32(0.7)
    got = ctx.update_w(v, vv, z, w, float(step))
    want = step * (np.float32(2) * vv - z) + (np.float32(1) - step) * w
    np.testing.assert_array_equal(got, want.astype(np.float32))


def test_invalid_arguments_do_not_poison_context(ctx):
    c = cases.get("single")
    bad = mtr.VolumeSize(0, 10, 0, 10, 0, 10, 9, 10, 10)  # X != Xend - Xstart
    with pytest.raises(mtr.MtrError) as e:
        ctx.wbp(c.axes[0], bad)
    assert e.value.status == mtr.ERR_INVALID_ARGUMENT
    a = mtr.AxisData(c.axes[0].x_coef.copy(), c.axes[0].y_coef, c.axes[0].data)
    a.x_coef[3] = np.nan
    with pytest.raises(mtr.MtrError):
        ctx.wbp(a, c.vol)
    # the context still works
    got = ctx.wbp(c.axes[0], c.vol)
    assert rel_l2(got, oracle.wbp(0, c.axes[0], c.vol)) < 1e-5


# --- the reference's own kernels (cubin built from FunctionOnGPU.cu) ------------------

needs_ref = pytest.mark.skipif(not oracle.refrun_available(), reason="reference cubin not built here")


@needs_ref
@pytest.mark.parametrize("name", ["single", "two_axis", "oob"])
def test_wbp_matches_reference_kernels(ctx, name):
    c = cases.get(name)
    a = c.axes[0]
    assert rel_l2(ctx.wbp(a, c.vol), oracle.ref_wbp(a, c.vol)) < 1e-5


@needs_ref
@pytest.mark.parametrize("name,no,ni,rho", [("single", 1, 10, 0.5), ("two_axis", 2, 3, 0.8)])
def test_reconstruct_matches_reference_kernels(ctx, name, no, ni, rho):
    c = cases.get(name)
    p = mtr.params(iter_times=no, sirt_inner=ni, sirt_step=0.5, mace_step=rho)
    got = ctx.reconstruct(c.axes, c.vol, p)
    want = oracle.ref_reconstruct(c.axes, c.vol, no, ni, 0.5, rho)
    assert rel_l2(got, want) < FP32_TOL


# --- TMA-windowed kernels (detector wide enough for the windowed forward) -----------

@pytest.mark.parametrize("name", ["mid", "mid_oblique"])
@pytest.mark.parametrize("prec", [mtr.PREC_FP32, mtr.PREC_MIXED_BF16])
def test_windowed_kernels_match_oracle(ctx, name, prec):
    c = cases.get(name)
    p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec)
    got = ctx.reconstruct(c.axes, c.vol, p)
    mode = oracle.REF_FAITHFUL if prec == mtr.PREC_FP32 else oracle.FP64
    want = oracle.reconstruct(mode, c.axes, c.vol, 2, 3, 0.5, 0.8)
    assert rel_l2(got, want) < (FP32_TOL if prec == mtr.PREC_FP32 else MIXED_TOL)


def test_windowed_kernels_z_dependent_y_map(ctx):
    c = cases.tilt_axis_in_z(cases.get("mid"))
    p = mtr.params(iter_times=1, sirt_inner=4, sirt_step=0.5, mace_step=0.7)
    got = ctx.reconstruct(c.axes, c.vol, p)
    want = oracle.reconstruct(oracle.REF_FAITHFUL, c.axes, c.vol, 1, 4, 0.5, 0.7)
    assert rel_l2(got, want) < FP32_TOL


def test_windowed_and_plain_kernels_agree(ctx, monkeypatch):
    c = cases.get("mid_oblique")
    p = mtr.params(iter_times=1, sirt_inner=3, sirt_step=0.5, mace_step=0.7)
    tma = ctx.reconstruct(c.axes, c.vol, p)
    monkeypatch.setenv("MTR_DISABLE_TMA", "1")
    plain = ctx.reconstruct(c.axes, c.vol, p)
    assert rel_l2(tma, plain) < 1e-5


# --- autotuned tile shapes: every depth variant is correct, the cache persists -------

@pytest.mark.parametrize("depths", ["4,8,0,0", "8,16,1,1", "16,32,0,1", "16,8,1,0", "8,32", "16,16,2,0", "4,8,2,1",
                                    "8,32,0,2", "16,8,2,2", "32,32,0,0", "32,16,2,1", "32,8,1,2",
                                    # the SIRT update over residual-pair windows
                                    "8,16,0,0,1", "16,32,2,1,1", "32,8,1,2,1", "4,16,2,0,1", "32,32,0,0,1",
                                    # ... over planar residual-pair windows
                                    "16,32,2,0,2", "8,16,0,1,2", "32,8,1,2,2", "4,32,2,2,2"])
@pytest.mark.parametrize("name", ["mid", "mid_oblique"])
def test_every_brick_depth_matches_oracle(ctx, monkeypatch, name, depths):
    monkeypatch.setenv("MTR_FORCE_DEPTHS", depths)
    c = cases.get(name)
    p = mtr.params(iter_times=1, sirt_inner=3, sirt_step=0.5, mace_step=0.7)
    got = ctx.reconstruct(c.axes, c.vol, p)
    want = oracle.reconstruct(oracle.REF_FAITHFUL, c.axes, c.vol, 1, 3, 0.5, 0.7)
    assert rel_l2(got, want) < FP32_TOL


# ... over FP16 residual-pair windows (mixed precision only; FP32 runs clamp
# the format to planar FP32 pairs)
@pytest.mark.parametrize("depths", ["16,32,2,0,3", "8,16,0,1,3", "32,8,1,2,3", "4,32,2,2,3", "32,32,0,0,3"])
@pytest.mark.parametrize("name", ["mid", "mid_oblique"])
def test_fp16_pair_windows_match_fp64_oracle(ctx, monkeypatch, name, depths):
    monkeypatch.setenv("MTR_FORCE_DEPTHS", depths)
    c = cases.get(name)
    p = mtr.params(iter_times=1, sirt_inner=3, sirt_step=0.5, mace_step=0.7, precision=mtr.PREC_MIXED_FP16)
    r = mtr.Recon(ctx, c.axes, c.vol, p)
    try:
        assert all(d["back_projection"]["window_format"] == "fp16 pairs" for d in r.describe())
        r.run()
        got = r.download()
    finally:
        r.close()
    want = oracle.reconstruct(oracle.FP64, c.axes, c.vol, 1, 3, 0.5, 0.7)
    assert rel_l2(got, want) < MIXED_TOL
    p32 = mtr.params(iter_times=1, sirt_inner=3, sirt_step=0.5, mace_step=0.7)
    got32 = ctx.reconstruct(c.axes, c.vol, p32)
    assert rel_l2(got32, oracle.reconstruct(oracle.REF_FAITHFUL, c.axes, c.vol, 1, 3, 0.5, 0.7)) < FP32_TOL


def test_fp16_pair_windows_z_dependent_y_map(ctx, monkeypatch):
    monkeypatch.setenv("MTR_FORCE_DEPTHS", "8,16,0,0,3")
    c = cases.tilt_axis_in_z(cases.get("mid"))
    p = mtr.params(iter_times=1, sirt_inner=4, sirt_step=0.5, mace_step=0.7, precision=mtr.PREC_MIXED_FP16)
    got = ctx.reconstruct(c.axes, c.vol, p)
    want = oracle.reconstruct(oracle.FP64, c.axes, c.vol, 1, 4, 0.5, 0.7)
    assert rel_l2(got, want) < MIXED_TOL


def test_autotune_cache_file(ctx, monkeypatch, tmp_path):
    import json

    cache = tmp_path / "tune.json"
    monkeypatch.setenv("MTR_AUTOTUNE_CACHE", str(cache))
    c = cases.get("mid")
    # a geometry not seen before in this process: shift the volume frame
    v = mtr.VolumeSize.make(c.vol.Xstart, c.vol.Xend, c.vol.Ystart, c.vol.Yend, 0, 19)
    p = mtr.params(iter_times=1, sirt_inner=2, sirt_step=0.5, mace_step=0.7)
    ctx.reconstruct(c.axes, v, p)
    d = json.loads(cache.read_text())
    # lane -1: no windowed candidate fits that detector (the plain kernel runs)
    assert d and all(b in (4, 8, 16, 32) and f in (8, 16, 32) and bl in (-1, 0, 1, 2) and fl in (-1, 0, 1, 2)
                     and bp in (0, 1, 2, 3) for b, f, bl, fl, bp in d.values())
    key = next(k for k in d if k.startswith("p72x72x13_v64x48x19"))
    assert d[key][2] in (0, 1, 2) and d[key][3] in (0, 1, 2)  # this detector fits both windowed kernels


# --- the all-FP64 GPU path used as the error reference at full sizes ---------------

@pytest.mark.parametrize("name", ["two_axis", "mid_oblique", "rect"])
def test_fp64_gpu_reference_matches_fp64_oracle(ctx, name):
    c = cases.get(name)
    p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8)
    got = ctx.reconstruct_fp64(c.axes, c.vol, p)
    want = oracle.reconstruct(oracle.FP64, c.axes, c.vol, 2, 3, 0.5, 0.8)
    # Two FP64 implementations: the GPU contracts the map evaluation into FMAs
    # and adds ray sums with double atomics in any order, which moves
    # near-zero-weight taps at the footprint edge (c == 0 vs c tiny); observed
    # ~1e-8, four to five orders below the errors this reference measures.
    assert rel_l2(got, want) < 1e-7


def test_entry_points_without_projection_data_are_rejected(ctx):
    """mtr_reconstruct and mtr_batch_create have no later upload, so an axis
    without projection data is an invalid argument (mtr_recon_create alone
    accepts it, for a later mtr_recon_upload)."""
    import ctypes as C

    c = cases.get("single")
    shape_only = [mtr.AxisData(a.x_coef, a.y_coef, tuple(a.data.shape)) for a in c.axes]
    arr = (mtr.AxisC * len(shape_only))(*[a.c_struct() for a in shape_only])
    out = np.empty(c.vol.shape, np.float32)
    p = mtr.params(iter_times=1, sirt_inner=1)
    st = ctx.lib.mtr_reconstruct(ctx.h, len(shape_only), arr, c.vol, C.byref(p), out.ctypes.data)
    assert st == mtr.ERR_INVALID_ARGUMENT
    inst = (mtr.InstanceC * 1)(mtr.InstanceC(len(shape_only), arr, c.vol))
    h = C.c_void_p()
    st = ctx.lib.mtr_batch_create(ctx.h, 1, inst, C.byref(p), mtr.MEM_HOST, C.byref(h))
    assert st == mtr.ERR_INVALID_ARGUMENT and not h.value
    # the context still works
    assert rel_l2(ctx.wbp(c.axes[0], c.vol), oracle.wbp(0, c.axes[0], c.vol)) < 1e-5


@pytest.mark.parametrize("name", ["mid", "mid_oblique"])
def test_reference_shaped_entry_points_run_windowed_kernels(ctx, name):
    """mtr_wbp / mtr_sirt (the calls that replace ComputeInitialModel and
    runSIRTOnGPU) run the TMA-windowed projectors where the windows fit, and
    keep the oracle's result."""
    c = cases.get(name)
    a = c.axes[0]
    n0 = ctx.windowed_launch_count()
    x0 = ctx.wbp(a, c.vol)
    n1 = ctx.windowed_launch_count()
    got = ctx.sirt(a, c.vol, x0, n_inner=3, step=0.5)
    n2 = ctx.windowed_launch_count()
    assert n1 - n0 >= 1  # the WBP gather
    assert n2 - n1 >= 1 + 2 * 3  # weight sums, then a forward splat and a back-projection per iteration
    assert rel_l2(x0, oracle.wbp(oracle.REF_FAITHFUL, a, c.vol)) < 1e-5
    want = oracle.sirt(oracle.REF_FAITHFUL, a, c.vol, x0, 3, 0.5)
    assert rel_l2(got, want) < FP32_TOL
