"""Record how the reference's own CPU code parses options, reads MRC stacks
and TXBR maps, and writes the output volume.

Runs oracle/_ref/ref_golden (built by oracle/build.py from the reference's
ReadAndInitialOptions.cpp, MrcFileIO.cpp and MrcFileIOBaseFunction.cpp) on
small inputs written here with numpy, and stores inputs + records under
tests/golden/io/.  Needs the reference sources (x86-64 build host).

    python tests/golden/make_golden_io.py
"""
from __future__ import annotations

import json
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "multi-tilt-reconstuction_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

import build as oracle_build  # noqa: E402  (oracle/build.py)
import phantom  # noqa: E402

OUT = Path(__file__).resolve().parent / "io"
GOLDEN_BIN = ROOT / "oracle" / "_ref" / "ref_golden"


def mrc_bytes(data: np.ndarray, mode: int) -> bytes:
    """Minimal MRC: 1024-byte header (nx, ny, nz, mode, ..., mapc/r/s) + data."""
    nz, ny, nx = data.shape
    h = bytearray(1024)
    struct.pack_into("<10i", h, 0, nx, ny, nz, mode, 0, 0, 0, nx, ny, nz)
    struct.pack_into("<6f", h, 40, nx, ny, nz, 90, 90, 90)
    struct.pack_into("<3i", h, 64, 1, 2, 3)
    h[208:212] = b"MAP "
    h[212:216] = b"DA\x00\x00"
    body = {1: data.astype("<i2"), 2: data.astype("<f4"), 6: data.astype("<u2")}[mode].tobytes()
    return bytes(h) + body


def run(*args) -> dict:
    r = subprocess.run([str(GOLDEN_BIN), *map(str, args)], capture_output=True, text=True, check=True)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("JSON:")][-1]
    return json.loads(line[5:])


# Inputs of the libmtr-written TXBR record (also used by tests/test_io.py).
TXBR_WRITTEN = dict(tilts=[-58.0, -41.5, -20.25, 0.0, 17.75, 39.0, 61.5], phi=37.5, det=(96, 80),
                    vol=(-10, 70, 3, 61, -6, 18),
                    xf=[[np.cos(0.02 * k), -np.sin(0.02 * k), np.sin(0.02 * k), np.cos(0.02 * k), 0.3 * k - 1.0,
                         -0.45 * k + 0.7] for k in range(7)])


class V:
    def __init__(self, xs, xe, ys, ye, zs, ze):
        self.Xstart, self.Xend, self.Ystart, self.Yend, self.Zstart, self.Zend = xs, xe, ys, ye, zs, ze


def main() -> None:
    oracle_build.build()
    OUT.mkdir(exist_ok=True)
    rng = np.random.default_rng(2024)
    rec = {}
    # --- mode-1 stack + TXBR map -----------------------------------------------------
    stack = rng.integers(-30000, 30000, size=(4, 12, 12)).astype(np.int16)
    (OUT / "stack_mode1.st").write_bytes(mrc_bytes(stack, 1))
    vol = V(-3, 9, 2, 14, 0, 5)
    xc, yc = phantom.axis_maps(12, 12, [-45.0, -15.0, 15.0, 45.0], 30.0, vol)
    (OUT / "map.txbr").write_text(phantom.txbr_text(xc, yc, vol))
    rec["read"] = run("read", OUT / "stack_mode1.st", OUT / "map.txbr")
    # a second map widening the bounds (the union is the reference's synchronizeVol)
    vol2 = V(-5, 7, 0, 16, -1, 4)
    (OUT / "map2.txbr").write_text(phantom.txbr_text(xc, yc, vol2))
    rec["read2"] = run("read", OUT / "stack_mode1.st", OUT / "map2.txbr")
    # trailing blank before the newline: the reference appends a spurious 0 coefficient
    (OUT / "map_trailing_blank.txbr").write_text(phantom.txbr_text(xc, yc, vol).replace("\n", " \n", 2))
    rec["read_trailing_blank"] = run("read", OUT / "stack_mode1.st", OUT / "map_trailing_blank.txbr")
    # a TXBR file written by libmtr (maps of a tilt series with 2-D alignments,
    # mtr_geometry_from_tilts) as the reference's readCoef parses it
    import mtr

    tw = TXBR_WRITTEN
    vw = mtr.VolumeSize.make(*tw["vol"])
    xw, yw = mtr.geometry_from_tilts(tw["tilts"], tw["phi"], tw["det"][0], tw["det"][1], vw, xf=tw["xf"])
    mtr.write_txbr(OUT / "written.txbr", xw, yw, vw)
    stack_w = np.random.default_rng(2025).integers(-30000, 30000, size=(len(tw["tilts"]), 12, 12)).astype(np.int16)
    (OUT / "stack_written.st").write_bytes(mrc_bytes(stack_w, 1))
    rec["read_written"] = run("read", OUT / "stack_written.st", OUT / "written.txbr")
    rec["read_written"].pop("data")
    # --- options --------------------------------------------------------------------
    rec["options"] = {
        "full": run("options", "MultiAxis", "-i", "2,a.st,b.st,a.txbr,b.txbr", "-o", "out.mrc", "-n", "3", "-s",
                    "0.25", "-m", "0.6", "-x", "4", "-y", "2", "-z", "16"),
        "defaults": run("options", "MultiAxis", "-i", "1,one.st,one.txbr", "-o", "o.mrc"),
        "help": run("options", "MultiAxis", "-h", "-i", "1,one.st,one.txbr", "-o", "o.mrc"),
        "invalid": run("options", "MultiAxis", "-q", "-o", "o.mrc"),
    }
    # --- output volume ---------------------------------------------------------------
    data = rng.normal(size=(3, 5, 6)).astype(np.float32)
    (OUT / "vol_data.f32").write_bytes(data.tobytes())
    rec["write"] = run("write", OUT / "ref_write.mrc", -2, 4, 1, 6, 7, 10, OUT / "vol_data.f32")
    (OUT / "ref_read.json").write_text(json.dumps(rec, indent=1))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
