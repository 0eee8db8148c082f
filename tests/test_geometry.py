"""Geometry front end (mtr_geometry_from_tilts, .tlt/.xf readers): the
identity alignment reproduces the synthetic tilt geometry the parity cases
use, an alignment transform inverts exactly, and the readers reject
malformed files."""
import numpy as np
import pytest

import mtr
import phantom


@pytest.mark.parametrize("phi", [0.0, 37.5, 90.0, 135.0])
@pytest.mark.parametrize("shape", [(96, 96, (0, 64, 0, 64, 0, 24)), (80, 64, (3, 70, -5, 41, 2, 19))])
def test_identity_alignment_is_the_tilt_geometry(phi, shape):
    px, py, v = shape
    vol = mtr.VolumeSize.make(*v)
    tilts = np.arange(-60, 61, 7.5)
    want_x, want_y = phantom.axis_maps(px, py, tilts, phi, vol)
    x, y = mtr.geometry_from_tilts(tilts, phi, px, py, vol)
    np.testing.assert_allclose(x, want_x, rtol=0, atol=1e-12)
    np.testing.assert_allclose(y, want_y, rtol=0, atol=1e-12)
    eye = np.tile([1.0, 0.0, 0.0, 1.0, 0.0, 0.0], (len(tilts), 1))
    x2, y2 = mtr.geometry_from_tilts(tilts, phi, px, py, vol, xf=eye)
    np.testing.assert_array_equal(x2, x)
    np.testing.assert_array_equal(y2, y)


def test_alignment_maps_raw_views():
    """raw = C + A^-1 (al - C - d): applying the transform to the raw
    coordinates the maps give returns the aligned coordinates."""
    rng = np.random.default_rng(7)
    vol = mtr.VolumeSize.make(0, 50, 0, 40, 0, 16)
    px, py = 64, 48
    tilts = np.linspace(-55, 55, 12)
    xf = np.empty((12, 6))
    for k in range(12):
        r = np.deg2rad(rng.uniform(-5, 5))
        m = rng.uniform(0.97, 1.03)
        xf[k] = [m * np.cos(r), -m * np.sin(r), m * np.sin(r), m * np.cos(r), rng.uniform(-6, 6), rng.uniform(-6, 6)]
    phi = 20.0
    x_al, y_al = mtr.geometry_from_tilts(tilts, phi, px, py, vol)
    x_raw, y_raw = mtr.geometry_from_tilts(tilts, phi, px, py, vol, xf=xf)
    C = np.array([(px + 1) / 2.0, (py + 1) / 2.0])
    pts = np.column_stack([rng.uniform(0, 50, 200), rng.uniform(0, 40, 200), rng.uniform(0, 16, 200), np.ones(200)])
    for k in range(12):
        def at(coef):
            c = coef[4 * k:4 * k + 4]
            return c[0] + pts[:, :3] @ c[1:]
        al = np.column_stack([at(x_al), at(y_al)])
        raw = np.column_stack([at(x_raw), at(y_raw)])
        A = xf[k, :4].reshape(2, 2)
        back = (raw - C) @ A.T + xf[k, 4:] + C
        np.testing.assert_allclose(back, al, rtol=0, atol=1e-9)


def test_invalid_geometry_is_rejected():
    vol = mtr.VolumeSize.make(0, 8, 0, 8, 0, 4)
    with pytest.raises(mtr.MtrError):
        mtr.geometry_from_tilts([0.0, 10.0], 0.0, 16, 16, vol, xf=[[1, 0, 0, 1, 0, 0], [1, 2, 0.5, 1, 0, 0]])
    with pytest.raises(mtr.MtrError):
        mtr.geometry_from_tilts([np.nan], 0.0, 16, 16, vol)
    with pytest.raises(mtr.MtrError):
        mtr.geometry_from_tilts([0.0], 0.0, 0, 16, vol)


def test_tlt_and_xf_files(tmp_path):
    tlt = tmp_path / "a.tlt"
    tlt.write_text("-60.0\n  -58.5\n\n0\n 61.25 \n")
    np.testing.assert_array_equal(mtr.read_tlt(tlt), [-60.0, -58.5, 0.0, 61.25])
    xf = tmp_path / "a.xf"
    rows = [[0.99, -0.01, 0.01, 0.99, 1.5, -2.25], [1, 0, 0, 1, 0, 0]]
    xf.write_text("\n".join("  ".join(f"{v:.7f}" for v in r) for r in rows) + "\n")
    np.testing.assert_allclose(mtr.read_xf(xf), rows, atol=1e-12)
    bad = tmp_path / "bad.xf"
    bad.write_text("1 0 0 1 0\n")
    with pytest.raises(mtr.MtrError) as e:
        mtr.read_xf(bad)
    assert e.value.status == mtr.ERR_FORMAT
    bad.write_text("1 0 0 1 0 zero\n")
    with pytest.raises(mtr.MtrError):
        mtr.read_xf(bad)
    with pytest.raises(mtr.MtrError) as e:
        mtr.read_tlt(tmp_path / "missing.tlt")
    assert e.value.status == mtr.ERR_IO


def test_maps_from_files_reconstruct_like_txbr(tmp_path):
    """A tilt series described by .tlt + .xf files yields the maps a TXBR file
    of the same geometry holds (read by the reference-grammar reader), and
    reconstructs (CPU oracle WBP) the same volume."""
    import oracle

    vol = mtr.VolumeSize.make(0, 32, 0, 32, 0, 12)
    tilts = np.arange(-60, 61, 10.0)
    xf = np.tile([np.cos(0.03), -np.sin(0.03), np.sin(0.03), np.cos(0.03), 0.75, -0.5], (len(tilts), 1))
    (tmp_path / "s.tlt").write_text("\n".join(f"{t:.3f}" for t in tilts))
    (tmp_path / "s.xf").write_text("\n".join(" ".join(f"{v:.12f}" for v in r) for r in xf))
    x, y = mtr.geometry_from_tilts(mtr.read_tlt(tmp_path / "s.tlt"), 0.0, 40, 40, vol, xf=mtr.read_xf(tmp_path / "s.xf"))
    ell = phantom.random_ellipsoids(np.random.default_rng(3), 6, vol)
    data = phantom.line_integrals(ell, x, y, 40, 40).astype(np.float32)
    a = mtr.AxisData(x, y, data)
    w = oracle.wbp(oracle.REF_FAITHFUL, a, vol)
    (tmp_path / "s.txbr").write_text(phantom.txbr_text(*mtr.geometry_from_tilts(tilts, 0.0, 40, 40, vol, xf=xf), vol))
    x0, y0, vol0 = mtr.read_txbr(tmp_path / "s.txbr", 4 * len(tilts))
    assert (vol0.X, vol0.Y, vol0.Z) == (vol.X, vol.Y, vol.Z)
    np.testing.assert_allclose(x0, x, rtol=0, atol=1e-9)
    np.testing.assert_allclose(y0, y, rtol=0, atol=1e-9)
    w0 = oracle.wbp(oracle.REF_FAITHFUL, mtr.AxisData(x0, y0, data), vol0)
    np.testing.assert_allclose(w, w0, rtol=1e-9, atol=1e-9)
    assert np.linalg.norm(w) > 0
