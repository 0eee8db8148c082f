"""MRC stacks read straight into device memory (mtr_mrc_read_stack_device)
give exactly the values of the host reader, for every supported mode and
across chunk boundaries; the half-precision reader gives those values
rounded to FP16, and FP16 projections uploaded into a reconstruction
(mtr_recon_upload_half) give the reconstruction of the same rounded data."""
import numpy as np
import pytest

import mtr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1, 2, 6, 12])
def test_device_read_equals_host_read(ctx, tmp_path, mode):
    import torch

    rng = np.random.default_rng(mode)
    lo, hi = {0: (0, 255), 1: (-30000, 30000), 2: (-1e3, 1e3), 6: (0, 65535), 12: (-100, 100)}[mode]
    data = rng.uniform(lo, hi, (7, 33, 45)).astype(np.float32)
    path = tmp_path / f"m{mode}.mrc"
    if mode in (0, 6):  # modes the writer does not produce: patch a mode-1 header
        mtr.write_mrc_stack(path, np.zeros_like(data), 1)
        hdr = bytearray(path.read_bytes()[:1024])
        hdr[12:16] = np.int32(mode).tobytes()
        raw = np.round(data).astype(np.uint8 if mode == 0 else np.uint16).tobytes()
        path.write_bytes(bytes(hdr) + raw)
    else:
        mtr.write_mrc_stack(path, data, mode)
    host = mtr.read_mrc_stack(path)
    dev = torch.empty(host.size, dtype=torch.float32, device="cuda")
    mtr.read_mrc_stack_device(ctx, path, dev)
    np.testing.assert_array_equal(dev.cpu().numpy().reshape(host.shape), host)


def test_device_read_spans_chunks(ctx, tmp_path):
    import torch

    # 48 Mi int16 values = 96 MiB: three 32 MiB chunks through two pinned buffers
    nz, ny, nx = 24, 1024, 2048
    data = (np.arange(nz * ny * nx, dtype=np.int64) % 60001 - 30000).astype(np.float32).reshape(nz, ny, nx)
    path = tmp_path / "big.mrc"
    mtr.write_mrc_stack(path, data, 1)
    dev = torch.empty(data.size, dtype=torch.float32, device="cuda")
    mtr.read_mrc_stack_device(ctx, path, dev)
    np.testing.assert_array_equal(dev.cpu().numpy().reshape(data.shape), data)


def test_device_read_errors(ctx, tmp_path):
    import torch

    dev = torch.empty(10, dtype=torch.float32, device="cuda")
    with pytest.raises(mtr.MtrError):
        mtr.read_mrc_stack_device(ctx, tmp_path / "missing.mrc", dev)
    path = tmp_path / "small.mrc"
    mtr.write_mrc_stack(path, np.zeros((1, 2, 2), np.float32), 1)
    big = torch.empty(100, dtype=torch.float32, device="cuda")
    with pytest.raises(mtr.MtrError) as e:
        mtr.read_mrc_stack_device(ctx, path, big)  # more values asked than the file holds
    assert e.value.status == mtr.ERR_FORMAT


@pytest.mark.parametrize("mode", [1, 2, 12])
def test_half_read_equals_host_read_rounded(ctx, tmp_path, mode):
    import torch

    rng = np.random.default_rng(10 + mode)
    lo, hi = {1: (-30000, 30000), 2: (-1e3, 1e3), 12: (-100, 100)}[mode]
    data = rng.uniform(lo, hi, (5, 31, 47)).astype(np.float32)
    path = tmp_path / f"h{mode}.mrc"
    mtr.write_mrc_stack(path, data, mode)
    host = mtr.read_mrc_stack(path)
    dev = torch.empty(host.size, dtype=torch.float16, device="cuda")
    mtr.read_mrc_stack_device_half(ctx, path, dev)
    got = dev.cpu().numpy().reshape(host.shape).view(np.uint16)
    np.testing.assert_array_equal(got, host.astype(np.float16).view(np.uint16))


@pytest.mark.parametrize("prec", [mtr.PREC_MIXED_BF16, mtr.PREC_FP32])
def test_half_upload_reconstructs_the_rounded_data(ctx, prec):
    import cases
    from conftest import rel_l2, run_to_run_tol

    c = cases.get("two_axis")
    p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec)
    halves = [np.ascontiguousarray(np.asarray(a.data, dtype=np.float32).astype(np.float16)) for a in c.axes]
    rounded = [mtr.AxisData(a.x_coef, a.y_coef, h.astype(np.float32)) for a, h in zip(c.axes, halves)]
    want = ctx.reconstruct(rounded, c.vol, p)
    deferred = [mtr.AxisData(a.x_coef, a.y_coef, tuple(np.shape(a.data))) for a in c.axes]
    r = mtr.Recon(ctx, deferred, c.vol, p)
    for k, h in enumerate(halves):
        r.upload_half(k, h)
    r.run()
    got = r.download()
    r.close()
    assert rel_l2(got, want) < run_to_run_tol(prec)
