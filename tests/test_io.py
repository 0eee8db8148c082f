"""MRC / TXBR / option parsing of libmtr against records of the reference's own
CPU code (tests/golden/io/, made by make_golden_io.py from
ReadAndInitialOptions.cpp, MrcFileIO.cpp and MrcFileIOBaseFunction.cpp)."""
import ctypes
import json
import struct
from pathlib import Path

import numpy as np
import pytest

import mtr
import phantom

IO = Path(__file__).parent / "golden" / "io"


@pytest.fixture(scope="module")
def rec():
    return json.loads((IO / "ref_read.json").read_text())


def test_mode1_stack_reads_like_reference(rec):
    r = rec["read"]
    h = mtr.read_mrc_header(str(IO / "stack_mode1.st"))
    assert (h.nx, h.nx, h.nz) == tuple(r["prj"])  # the reference sets prj.Y = nx (MrcFileIO.cpp:121)
    assert h.mode == r["mode"] == 1
    data = mtr.read_mrc_stack(str(IO / "stack_mode1.st"))
    np.testing.assert_array_equal(data.reshape(-1), np.array(r["data"], np.float32))


def test_txbr_reads_like_reference(rec):
    r = rec["read"]
    x, y, vol = mtr.read_txbr(str(IO / "map.txbr"), 4 * 4)
    np.testing.assert_array_equal(x, np.array(r["x_coef"]))
    np.testing.assert_array_equal(y, np.array(r["y_coef"]))
    assert list(vol.astuple()) == r["vol"]


def test_txbr_bounds_union_over_axes(rec):
    _, _, vol = mtr.read_txbr(str(IO / "map.txbr"), 16)
    _, _, vol = mtr.read_txbr(str(IO / "map2.txbr"), 16, vol)
    a, b = rec["read"]["vol"], rec["read2"]["vol"]
    want = [min(a[0], b[0]), max(a[1], b[1]), min(a[2], b[2]), max(a[3], b[3]), min(a[4], b[4]), max(a[5], b[5])]
    assert list(vol.astuple())[:6] == want
    assert (vol.X, vol.Y, vol.Z) == (want[1] - want[0], want[3] - want[2], want[5] - want[4])


def test_txbr_trailing_blank_is_not_a_coefficient(rec):
    # The reference appends a spurious 0 after a blank before the newline
    # (strtok on ' ' then strtod("\n")); libmtr reads the intended values.
    ref = rec["read_trailing_blank"]["x_coef"]
    assert ref[4] == 0.0 and rec["read"]["x_coef"][4] != 0.0
    x, _, _ = mtr.read_txbr(str(IO / "map_trailing_blank.txbr"), 16)
    np.testing.assert_array_equal(x, np.array(rec["read"]["x_coef"]))


@pytest.mark.parametrize("case", ["full", "defaults"])
def test_options_match_reference(rec, case):
    r = rec["options"][case]
    argv = {"full": ["MultiAxis", "-i", "2,a.st,b.st,a.txbr,b.txbr", "-o", "out.mrc", "-n", "3", "-s", "0.25", "-m",
                     "0.6", "-x", "4", "-y", "2", "-z", "16"],
            "defaults": ["MultiAxis", "-i", "1,one.st,one.txbr", "-o", "o.mrc"]}[case]
    st, o = mtr.parse_options(argv)
    assert st == 0 and r["rc"] == 1
    assert o.number_tilt == r["number_tilt"]
    assert [o.block_x, o.block_y, o.block_z] == r["block"]
    assert o.iter_times == r["iter_times"]
    assert np.float32(o.sirt_step) == np.float32(r["sirt_step"])
    assert np.float32(o.mace_step) == np.float32(r["mace_step"])
    assert o.out_path.decode() == r["out"]
    assert [o.mrc_path[i].value.decode() for i in range(o.number_tilt)] == r["mrc"]
    assert [o.txbr_path[i].value.decode() for i in range(o.number_tilt)] == r["txbr"]
    assert o.sirt_inner == 10 and o.precision == 0


def test_options_help_and_invalid(rec):
    # reference: -h prints help and returns 0 (the caller carries on); invalid -> -1 (ignored by main)
    assert rec["options"]["help"]["rc"] == 0 and rec["options"]["invalid"]["rc"] == -1
    st, o = mtr.parse_options(["MultiAxis", "-h"])
    assert st == 0 and o.help == 1
    st, _ = mtr.parse_options(["MultiAxis", "-q", "-o", "o.mrc"])
    assert st == mtr.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("argv", [["p", "-i", "2,a.st,a.txbr"], ["p", "-i", "0"], ["p", "-i", "17" + ",a" * 34],
                                  ["p", "-n", "x"], ["p", "-s"], ["p", "-i", "1,a.st,a.txbr", "extra"],
                                  ["p", "--precision", "fp8"], ["p", "--inner", "-1"]])
def test_options_errors(argv):
    st, _ = mtr.parse_options(argv)
    assert st == mtr.ERR_INVALID_ARGUMENT


def test_options_long_only():
    st, o = mtr.parse_options(["p", "-i", "1,a.st,a.txbr", "-o", "o", "--inner", "7", "--precision", "bf16"])
    assert st == 0 and o.sirt_inner == 7 and o.precision == mtr.PREC_MIXED_BF16
    # repeated calls start from a clean parser state
    st, o = mtr.parse_options(["p", "-n", "2"])
    assert st == 0 and o.iter_times == 2 and o.number_tilt == 0


def test_output_volume_matches_reference(tmp_path):
    ref = (IO / "ref_write.mrc").read_bytes()
    data = np.frombuffer((IO / "vol_data.f32").read_bytes(), np.float32).reshape(3, 5, 6)
    vol = mtr.VolumeSize.make(-2, 4, 1, 6, 7, 10)
    out = tmp_path / "o.mrc"
    mtr.write_mrc_volume(str(out), vol, data)
    got = out.read_bytes()
    assert len(got) == len(ref) == 1024 + data.nbytes
    assert got[1024:] == ref[1024:]  # data block, x fastest
    # header fields the reference sets (MrcFileIO.cpp:3-88)
    for off, fmt in [(0, "<10i"), (40, "<6f"), (64, "<3i"), (76, "<3f"), (88, "<2h"), (92, "<i"), (96, "<h")]:
        assert struct.unpack_from(fmt, got, off) == struct.unpack_from(fmt, ref, off), off
    assert got[208:211] == ref[208:211] == b"MAP" and got[212:213] == ref[212:213] == b"D"


def test_mrc_round_trip_modes(tmp_path):
    rng = np.random.default_rng(1)
    d = rng.integers(-2000, 2000, size=(3, 7, 5)).astype(np.float32)
    for mode in (1, 2, 12):
        p = tmp_path / f"s{mode}.mrc"
        mtr.write_mrc_stack(str(p), d, mode)
        h = mtr.read_mrc_header(str(p))
        assert (h.nx, h.ny, h.nz, h.mode) == (5, 7, 3, mode)
        np.testing.assert_array_equal(mtr.read_mrc_stack(str(p)), d)  # integers < 2048 are exact in fp16


def test_mrc_mode0_and_6(tmp_path):
    d = np.arange(24, dtype=np.uint16).reshape(2, 3, 4)
    for mode, dt in ((0, np.uint8), (6, "<u2")):
        h = bytearray(1024)
        struct.pack_into("<4i", h, 0, 4, 3, 2, mode)
        p = tmp_path / f"m{mode}.mrc"
        p.write_bytes(bytes(h) + b"\x00" * 16 + d.astype(dt).tobytes())  # extended header ignored: data is at the end
        np.testing.assert_array_equal(mtr.read_mrc_stack(str(p)), d.astype(np.float32))


def test_mrc_errors(tmp_path):
    lib = mtr.load()
    out = np.zeros(10, np.float32)
    assert lib.mtr_mrc_read_stack(b"/nonexistent/x.mrc", out.ctypes.data, 10) == mtr.ERR_IO
    short = tmp_path / "short.mrc"
    short.write_bytes(b"\x00" * 100)
    h = mtr.MrcHeader()
    assert lib.mtr_mrc_read_header(str(short).encode(), ctypes.byref(h)) == mtr.ERR_FORMAT
    trunc = tmp_path / "trunc.mrc"
    hb = bytearray(1024)
    struct.pack_into("<4i", hb, 0, 10, 10, 10, 1)
    trunc.write_bytes(bytes(hb) + b"\x00" * 50)
    big = np.zeros(1000, np.float32)
    assert lib.mtr_mrc_read_stack(str(trunc).encode(), big.ctypes.data, 1000) == mtr.ERR_FORMAT
    bad = tmp_path / "badmode.mrc"
    struct.pack_into("<4i", hb, 0, 1, 1, 1, 99)
    bad.write_bytes(bytes(hb) + b"\x00" * 8)
    assert lib.mtr_mrc_read_stack(str(bad).encode(), big.ctypes.data, 1) == mtr.ERR_UNSUPPORTED


@pytest.mark.parametrize("text", ["x-0: 1.0 abc 2.0\n", "x->5:1\n", "y->a:1:b\n"])
def test_txbr_malformed(tmp_path, text):
    p = tmp_path / "bad.txbr"
    p.write_text(text)
    with pytest.raises(mtr.MtrError) as e:
        mtr.read_txbr(str(p), 8)
    assert e.value.status == mtr.ERR_FORMAT


def test_txbr_capacity(tmp_path):
    vol = mtr.VolumeSize.make(0, 4, 0, 4, 0, 2)
    xc, yc = phantom.axis_maps(8, 8, [0.0, 10.0], 0.0, vol)
    p = tmp_path / "m.txbr"
    p.write_text(phantom.txbr_text(xc, yc, vol))
    with pytest.raises(mtr.MtrError) as e:
        mtr.read_txbr(str(p), 4)
    assert e.value.status == mtr.ERR_CAPACITY


def test_txbr_writer_round_trip(tmp_path):
    vol = mtr.VolumeSize.make(-7, 25, 3, 19, -2, 6)
    xc, yc = phantom.axis_maps(40, 36, np.arange(-60, 61, 30.0), 75.0, vol)
    p = tmp_path / "m.txbr"
    p.write_text(phantom.txbr_text(xc, yc, vol))
    x, y, v = mtr.read_txbr(str(p), len(xc))
    np.testing.assert_array_equal(x, xc)
    np.testing.assert_array_equal(y, yc)
    assert v.astuple() == vol.astuple()


def _written_inputs():
    """Inputs of the libmtr-written TXBR record (make_golden_io.TXBR_WRITTEN)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden_io", Path(__file__).parent / "golden" / "make_golden_io.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.TXBR_WRITTEN


def test_txbr_written_by_libmtr_is_read_by_the_reference_exactly(rec, tmp_path):
    """Maps of a tilt series with 2-D alignments (mtr_geometry_from_tilts),
    written by mtr_txbr_write: the reference's readCoef read the committed file
    (its record) back to exactly these coefficients and bounds, and libmtr
    still writes that file byte for byte."""
    tw = _written_inputs()
    vol = mtr.VolumeSize.make(*tw["vol"])
    xc, yc = mtr.geometry_from_tilts(tw["tilts"], tw["phi"], tw["det"][0], tw["det"][1], vol, xf=tw["xf"])
    p = tmp_path / "w.txbr"
    mtr.write_txbr(p, xc, yc, vol)
    assert p.read_bytes() == (IO / "written.txbr").read_bytes()
    r = rec["read_written"]
    assert r["read_rc"] == 1 and r["prj"][2] == len(tw["tilts"])
    np.testing.assert_array_equal(np.array(r["x_coef"]), xc)
    np.testing.assert_array_equal(np.array(r["y_coef"]), yc)
    assert tuple(r["vol"]) == vol.astuple()
    x, y, v = mtr.read_txbr(str(p), len(xc))  # and libmtr's reader agrees
    np.testing.assert_array_equal(x, xc)
    assert v.astuple() == vol.astuple()


def test_cli_converts_tilts_and_alignments_to_txbr(tmp_path):
    tw = _written_inputs()
    (tmp_path / "s.tlt").write_text("\n".join(repr(t) for t in tw["tilts"]) + "\n")
    (tmp_path / "s.xf").write_text("\n".join(" ".join(repr(float(v)) for v in row) for row in tw["xf"]) + "\n")
    cli = mtr.PKG / "bin" / "mtr_multiaxis"
    import subprocess

    args = [str(cli), "tilts2txbr", str(tmp_path / "s.tlt"), str(tmp_path / "o.txbr"), *map(str, tw["det"]),
            *map(str, tw["vol"]), repr(tw["phi"]), str(tmp_path / "s.xf")]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "o.txbr").read_bytes() == (IO / "written.txbr").read_bytes()
    r = subprocess.run([str(cli), "tilts2txbr", str(tmp_path / "s.tlt")], capture_output=True, text=True)
    assert r.returncode != 0


def test_txbr_writer_rejects_bad_input(tmp_path):
    vol = mtr.VolumeSize.make(0, 4, 0, 4, 0, 2)
    with pytest.raises(mtr.MtrError):
        mtr.write_txbr(tmp_path / "x.txbr", [np.nan, 1, 0, 0], [0, 0, 1, 0], vol)
    with pytest.raises(mtr.MtrError):
        mtr.write_txbr(tmp_path / "x.txbr", [0, 1, 0, 0], [0, 0, 1, 0], mtr.VolumeSize.make(0, 0, 0, 4, 0, 2))
