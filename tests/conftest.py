import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "multi-tilt-reconstuction_gb300"
for p in (ROOT, PKG, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built():
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import mtr

    c = mtr.Context(0)
    yield c
    c.close()


def run_to_run_tol(precision: int) -> float:
    """Bound for two runs of the same reconstruction.  The forward splat's
    float bulk reductions add in a run-dependent order (~1e-7 per iteration);
    in mixed precision such a difference now and then flips the BF16/FP16
    rounding of the volume copy the next forward reads (a 2^-9 step), which
    lifts run-to-run differences to ~1e-5 -- still 10x below the 1e-3 accuracy
    bound of the mixed path."""
    return 1e-5 if precision == 0 else 1e-4


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))
