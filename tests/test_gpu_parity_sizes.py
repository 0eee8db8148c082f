"""GPU parity at the benchmark configurations' geometries.

The small cases in cases.py pin the arithmetic; these pin it where precision
is stressed: the detector sizes, tilt counts and axis angles of the three
single-reconstruction workloads.
  c1  the whole single-axis workload: 128x128x32, 61 tilts (+-60 step 2),
      128^2 px, WBP + 10 SIRT at lambda 0.5 (rho 0.5 = plain SIRT);
  c2  the 3-axis geometry (512^2 px, 61 tilts, axes 0/60/120 deg) on a
      12-plane Z-slab of the 512x512x128 volume, 1 MACE x 2 SIRT;
  c3  the 4-axis geometry (2048^2 px, 121 tilts +-60 step 1, axes
      0/45/90/135 deg, Poisson dose 50) on a 256x256x8 crop at the far corner
      of the 2048x2048x256 volume, where detector coordinates reach ~2000 px
      and the FP64-base / FP32-offset tap coordinates are furthest from the
      reference's all-FP64 evaluation (FunctionOnGPU.cu:12-25), 1 MACE x 2 SIRT.
Each is compared with the reference-faithful oracle (FP32 path, 1e-4), the
all-FP64 oracle (mixed path, 1e-3) and, where the prebuilt cubin is present,
the reference's own kernels (FP32 path, 1e-4).  Every projection map is the
one of the full benchmark volume; the slab or crop is the reconstruction
frame, as a Z-slab rank of the reference reconstructs its part of the
volume with the whole volume's maps (MultiAxis.cpp:13-31)."""
import json
import os

import numpy as np
import pytest

import mtr
import oracle
import phantom
from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-4
MIXED_TOL = 1e-3

SIZES = {
    "c1": dict(frame=(0, 128, 0, 128, 0, 32), recon=(0, 128, 0, 128, 0, 32), px=128, tilts=(-60, 61, 2),
               phis=(0.0,), n_ell=20, noise=("gaussian", 0.02), seed=1001, no=1, ni=10, lam=0.5, rho=0.5),
    "c2": dict(frame=(0, 512, 0, 512, 0, 128), recon=(0, 512, 0, 512, 58, 70), px=512, tilts=(-60, 61, 2),
               phis=(0.0, 60.0, 120.0), n_ell=50, noise=("gaussian", 0.05), seed=1002, no=1, ni=2, lam=0.5,
               rho=0.8),
    "c3": dict(frame=(0, 2048, 0, 2048, 0, 256), recon=(1664, 1920, 1536, 1792, 124, 132), px=2048,
               tilts=(-60, 61, 1), phis=(0.0, 45.0, 90.0, 135.0), n_ell=200, noise=("poisson", 50.0), seed=1003,
               no=1, ni=2, lam=0.5, rho=0.7),
}


def _inputs(spec):
    import torch

    frame = mtr.VolumeSize.make(*spec["frame"])
    kind, level = spec["noise"]
    c = phantom.make_case_torch(frame, spec["px"], np.arange(*spec["tilts"], dtype=np.float64), list(spec["phis"]),
                                spec["n_ell"], kind, level, spec["seed"], device="cuda")
    axes = [mtr.AxisData(xc, yc, d.cpu().numpy()) for xc, yc, d in c["axes"]]
    del c
    torch.cuda.empty_cache()
    return axes, mtr.VolumeSize.make(*spec["recon"])


def _record(name, errs):
    """Error figures of the run, printed (and kept beside a GPU run's output
    when MTR_PARITY_RECORD names a file)."""
    print(f"parity[{name}] " + json.dumps(errs))
    path = os.environ.get("MTR_PARITY_RECORD")
    if path:
        rec = json.load(open(path)) if os.path.exists(path) else {}
        rec[name] = errs
        with open(path, "w") as f:
            json.dump(rec, f, indent=1)


@pytest.mark.parametrize("name", ["c1", "c2", "c3"])
def test_benchmark_geometry_parity(ctx, name):
    spec = SIZES[name]
    axes, vol = _inputs(spec)
    no, ni, lam, rho = spec["no"], spec["ni"], spec["lam"], spec["rho"]
    oracle.set_threads(os.cpu_count() or 1)
    p32 = mtr.params(iter_times=no, sirt_inner=ni, sirt_step=lam, mace_step=rho)
    pmx = mtr.params(iter_times=no, sirt_inner=ni, sirt_step=lam, mace_step=rho, precision=mtr.PREC_MIXED_BF16)
    pmh = mtr.params(iter_times=no, sirt_inner=ni, sirt_step=lam, mace_step=rho, precision=mtr.PREC_MIXED_FP16)
    got32 = ctx.reconstruct(axes, vol, p32)
    gotmx = ctx.reconstruct(axes, vol, pmx)
    gotmh = ctx.reconstruct(axes, vol, pmh)
    want = oracle.reconstruct(oracle.REF_FAITHFUL, axes, vol, no, ni, lam, rho)
    want64 = oracle.reconstruct(oracle.FP64, axes, vol, no, ni, lam, rho)
    errs = {"fp32_vs_oracle": rel_l2(got32, want), "mixed_bf16_vs_fp64_oracle": rel_l2(gotmx, want64),
            "mixed_fp16_vs_fp64_oracle": rel_l2(gotmh, want64),
            "fp32_vs_fp64_oracle": rel_l2(got32, want64), "oracle_vs_fp64_oracle": rel_l2(want, want64),
            "volume": list(vol.astuple()), "detector_px": spec["px"], "tilts": len(range(*spec["tilts"])),
            "axes_deg": list(spec["phis"])}
    if oracle.refrun_available():
        errs["fp32_vs_reference_kernels"] = rel_l2(got32, oracle.ref_reconstruct(axes, vol, no, ni, lam, rho))
    _record(name, errs)
    assert errs["fp32_vs_oracle"] < FP32_TOL
    assert errs["mixed_bf16_vs_fp64_oracle"] < MIXED_TOL
    assert errs["mixed_fp16_vs_fp64_oracle"] < MIXED_TOL
    if "fp32_vs_reference_kernels" in errs:
        assert errs["fp32_vs_reference_kernels"] < FP32_TOL
