"""Checkpoint / resume of the MACE state (mtr_recon_save / mtr_recon_load):
a run interrupted after an outer iteration and resumed in a fresh
reconstruction object equals the uninterrupted run, within the bound two
identical runs already keep (run_to_run_tol)."""
import numpy as np
import pytest

import cases
import mtr
from conftest import rel_l2, run_to_run_tol

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [mtr.PREC_FP32, mtr.PREC_MIXED_BF16])
def test_resume_equals_uninterrupted(ctx, tmp_path, prec):
    c = cases.get("two_axis")
    p = mtr.params(iter_times=3, sirt_inner=4, sirt_step=0.5, mace_step=0.8, precision=prec)
    straight = mtr.Recon(ctx, c.axes, c.vol, p)
    straight.run()
    want = straight.download()
    straight.close()
    # pieces: init + run_outer is the same run
    pieces = mtr.Recon(ctx, c.axes, c.vol, p)
    pieces.init()
    pieces.run_outer(0, 1)
    pieces.save(tmp_path / "after1.ckpt")
    pieces.run_outer(1, 2)
    assert rel_l2(pieces.download(), want) < run_to_run_tol(prec)
    pieces.close()
    resumed = mtr.Recon(ctx, c.axes, c.vol, p)
    done = resumed.load(tmp_path / "after1.ckpt")
    assert done == 1
    resumed.run_outer(done, 3 - done)
    assert rel_l2(resumed.download(), want) < run_to_run_tol(prec)
    resumed.close()


def test_checkpoint_of_another_volume_is_rejected(ctx, tmp_path):
    a, b = cases.get("two_axis"), cases.get("mid")
    p = mtr.params(iter_times=1, sirt_inner=1)
    r = mtr.Recon(ctx, a.axes, a.vol, p)
    r.run()
    r.save(tmp_path / "a.ckpt")
    r.close()
    other = mtr.Recon(ctx, b.axes, b.vol, p)
    with pytest.raises(mtr.MtrError) as e:
        other.load(tmp_path / "a.ckpt")
    assert e.value.status == mtr.ERR_INVALID_ARGUMENT
    data = (tmp_path / "a.ckpt").read_bytes()
    (tmp_path / "short.ckpt").write_bytes(data[: len(data) // 2])
    r2 = mtr.Recon(ctx, a.axes, a.vol, p)
    with pytest.raises(mtr.MtrError) as e:
        r2.load(tmp_path / "short.ckpt")
    assert e.value.status == mtr.ERR_FORMAT
    (tmp_path / "junk.ckpt").write_bytes(b"not a checkpoint" * 4)
    with pytest.raises(mtr.MtrError) as e:
        r2.load(tmp_path / "junk.ckpt")
    assert e.value.status == mtr.ERR_FORMAT
    r2.close()
    other.close()


def test_checkpoint_file_layout(ctx, tmp_path):
    c = cases.get("mid")
    r = mtr.Recon(ctx, c.axes, c.vol, mtr.params(iter_times=1, sirt_inner=2))
    r.run()
    r.save(tmp_path / "m.ckpt")
    wavg = r.download()
    r.close()
    raw = (tmp_path / "m.ckpt").read_bytes()
    assert raw[:8] == b"MTRCKPT1"
    hdr = np.frombuffer(raw[8:36], np.int32)
    assert list(hdr[:6]) == [1, len(c.axes), c.vol.X, c.vol.Y, c.vol.Z, 1]
    body = np.frombuffer(raw[48:], np.float32)
    n = c.vol.X * c.vol.Y * c.vol.Z
    assert body.size == n * (1 + len(c.axes))
    np.testing.assert_array_equal(body[:n].reshape(wavg.shape), wavg)


def test_convergence_record_and_early_stop(ctx):
    """mtr_recon_changes is the relative L2 change of the consensus per outer
    iteration (FP64 on the GPU); mtr_recon_run_until stops on it."""
    c = cases.get("two_axis")
    p = mtr.params(iter_times=4, sirt_inner=3, sirt_step=0.5, mace_step=0.8)
    plain = mtr.Recon(ctx, c.axes, c.vol, p)  # no record kept unless asked for
    with pytest.raises(mtr.MtrError):
        plain.changes(4)
    plain.close()
    pr = mtr.params(iter_times=4, sirt_inner=3, sirt_step=0.5, mace_step=0.8, flags=mtr.FLAG_RECORD_CHANGES)
    r = mtr.Recon(ctx, c.axes, c.vol, pr)
    r.init()
    vols = [r.download().astype(np.float64)]  # the WBP init consensus
    for it in range(4):
        r.run_outer(it, 1)
        vols.append(r.download().astype(np.float64))
    ch = r.changes(4)
    want = [np.linalg.norm(vols[i + 1] - vols[i]) / np.linalg.norm(vols[i + 1]) for i in range(4)]
    np.testing.assert_allclose(ch, want, rtol=1e-9)
    assert ch[0] > ch[1] > ch[2]
    r.close()
    for tol, expect in ((0.0, 4), (1e9, 1), (ch[1] * 1.001, 2)):
        r2 = mtr.Recon(ctx, c.axes, c.vol, p)
        r2.init()
        assert r2.run_until(tol) == expect
        r2.close()


@pytest.mark.parametrize("prec", [mtr.PREC_FP32, mtr.PREC_MIXED_BF16])
def test_host_resident_volumes(ctx, prec):
    """MTR_FLAG_HOST_VOLUMES: the volume arrays live in mapped host memory
    that the kernels read and write directly; the result is the device-resident one."""
    c = cases.get("two_axis")
    p = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec)
    dev = mtr.Recon(ctx, c.axes, c.vol, p)
    dev.run()
    want = dev.download()
    dev_bytes = dev.footprint()
    dev.close()
    ph = mtr.params(iter_times=2, sirt_inner=3, sirt_step=0.5, mace_step=0.8, precision=prec,
                    flags=mtr.FLAG_HOST_VOLUMES | mtr.FLAG_GRAPH)
    host = mtr.Recon(ctx, c.axes, c.vol, ph)
    host.run()
    got = host.download()
    assert host.footprint() < dev_bytes  # only the projections are in device memory
    host.close()
    assert rel_l2(got, want) < run_to_run_tol(prec)
