"""Small seeded reconstruction cases shared by the CPU and GPU tests and the
golden-vector generators.  Sizes are chosen so the CPU oracle finishes each
in well under a second."""
from __future__ import annotations

import numpy as np

import mtr
import phantom

CASES = {
    # one axis, volume frame not at the origin, coarse tilt series
    "single": dict(vol=(3, 27, 0, 20, 0, 8), px=28, py=None, tilts=(-60, 61, 15), phis=(0.0,), n_ell=5,
                   noise=("gaussian", 0.02), seed=11),
    # two axes, negative Y start
    "two_axis": dict(vol=(0, 20, -2, 22, 0, 6), px=26, py=None, tilts=(-60, 61, 20), phis=(0.0, 60.0), n_ell=6,
                     noise=("gaussian", 0.05), seed=12),
    # volume wider than the detector footprint: many taps fall off the detector, some voxels see none
    "oob": dict(vol=(0, 40, 0, 40, 0, 6), px=24, py=None, tilts=(-60, 61, 30), phis=(45.0,), n_ell=4,
                noise=("gaussian", 0.02), seed=13),
    # four axes at 0/45/90/135 degrees with Poisson noise
    "four_axis": dict(vol=(0, 16, 0, 16, 0, 5), px=20, py=None, tilts=(-60, 61, 30), phis=(0.0, 45.0, 90.0, 135.0),
                      n_ell=5, noise=("poisson", 50.0), seed=14),
    # detector wide enough for the windowed (TMA) forward splat; axes at 0 and 90 degrees
    "mid": dict(vol=(-8, 56, 4, 52, 0, 20), px=72, py=None, tilts=(-60, 61, 10), phis=(0.0, 90.0), n_ell=6,
                noise=("gaussian", 0.02), seed=16),
    # oblique axes with a ragged volume (no dimension a multiple of the brick)
    "mid_oblique": dict(vol=(0, 45, 0, 37, 0, 19), px=68, py=None, tilts=(-60, 61, 15), phis=(60.0, 135.0), n_ell=6,
                        noise=("gaussian", 0.05), seed=17),
}

# Non-square detector: supported by the product and the oracle (the reference
# reads prj.Y = nx, MrcFileIO.cpp:121, so it only handles square stacks).
RECT = dict(vol=(0, 18, 0, 14, 0, 7), px=30, py=22, tilts=(-50, 51, 25), phis=(30.0,), n_ell=4,
            noise=("gaussian", 0.02), seed=15)


def make(spec: dict) -> phantom.Case:
    vol = mtr.VolumeSize.make(*spec["vol"])
    tilts = np.arange(*spec["tilts"], dtype=np.float64)
    kind, level = spec["noise"]
    return phantom.make_case(vol, spec["px"], tilts, list(spec["phis"]), spec["n_ell"], kind, level, spec["seed"],
                             axis_cls=mtr.AxisData, py=spec["py"])


def get(name: str) -> phantom.Case:
    return make(RECT if name == "rect" else CASES[name])


def tilt_axis_in_z(case: phantom.Case, slope: float = 0.04) -> phantom.Case:
    """Give every y-map a Z term (a tilt axis not parallel to the XY plane)."""
    axes = []
    for a in case.axes:
        yc = a.y_coef.copy()
        yc[3::4] += slope
        axes.append(mtr.AxisData(a.x_coef, yc, a.data))
    return phantom.Case(case.vol, axes, case.ellipsoids, case.meta)
