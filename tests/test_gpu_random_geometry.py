"""Seeded random geometries through the tuned kernels: random in-plane axis
angles, tilt ranges and counts, ragged volume frames (negative starts,
sizes not multiples of any brick), non-square detectors and, for some,
tilt axes with a Z component.  Whatever warp layout, brick depth and window
pitch the tuner picks, the FP32 path stays within the FP32 bound of the
reference-faithful oracle and the mixed path within the mixed bound."""
import numpy as np
import pytest

import cases
import mtr
import oracle
import phantom
from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP32_TOL, MIXED_TOL = 1e-4, 1e-3


def random_case(seed: int):
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(v) for v in rng.integers([20, 20, 5], [70, 70, 24]))
    x0, y0, z0 = (int(v) for v in rng.integers(-10, 10, 3))
    vol = mtr.VolumeSize.make(x0, x0 + nx, y0, y0 + ny, z0, z0 + nz)
    px = int(max(nx, ny) + rng.integers(4, 20))
    py = int(px - rng.integers(0, 10))
    span = float(rng.uniform(40, 65))
    n = int(rng.integers(7, 16))
    tilts = np.linspace(-span, span, n)
    k = int(rng.integers(1, 4))
    phis = sorted(float(v) for v in rng.uniform(0, 180, k))
    case = phantom.make_case(vol, px, tilts, phis, 5, "gaussian", 0.02, 1000 + seed, axis_cls=mtr.AxisData, py=py)
    if seed % 3 == 0:
        case = cases.tilt_axis_in_z(case, 0.03)
    return case


@pytest.mark.parametrize("seed", range(6))
def test_random_geometry_matches_oracle(ctx, seed):
    c = random_case(seed)
    want = oracle.reconstruct(oracle.REF_FAITHFUL, c.axes, c.vol, 1, 3, 0.5, 0.7)
    got = ctx.reconstruct(c.axes, c.vol, mtr.params(iter_times=1, sirt_inner=3, sirt_step=0.5, mace_step=0.7))
    assert rel_l2(got, want) < FP32_TOL
    mixed = ctx.reconstruct(c.axes, c.vol, mtr.params(iter_times=1, sirt_inner=3, sirt_step=0.5, mace_step=0.7,
                                                       precision=mtr.PREC_MIXED_BF16))
    assert rel_l2(mixed, want) < MIXED_TOL
