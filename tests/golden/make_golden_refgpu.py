"""Record golden outputs of the reference's OWN CUDA kernels.

Runs FunctionOnGPU.cu's kernels (compiled unmodified into
oracle/_ref/ref_kernels.cubin) through oracle/ref_runner.cu, which restates
the reference's host logic with one rank per axis, on the small seeded cases
of tests/cases.py.  Needs a GPU; writes tests/golden/ref_gpu.npz (inputs and
outputs, float32) which the CPU tests compare the oracle against.

    python tests/golden/make_golden_refgpu.py [out.npz]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT, ROOT / "multi-tilt-reconstuction_gb300", ROOT / "oracle", ROOT / "tests"):
    sys.path.insert(0, str(p))

import cases  # noqa: E402
import oracle  # noqa: E402

# (case, n_outer, n_inner, sirt_step, mace_step)
RUNS = [("single", 1, 4, 0.5, 0.5), ("two_axis", 2, 3, 0.5, 0.8), ("oob", 1, 3, 0.5, 0.7),
        ("four_axis", 2, 2, 0.5, 0.7)]


def main(out: Path) -> None:
    rec = {}
    for name, no, ni, ls, rho in RUNS:
        c = cases.get(name)
        v = c.vol
        rec[f"{name}/vol"] = np.array(v.astuple(), np.int32)
        rec[f"{name}/params"] = np.array([no, ni, ls, rho], np.float64)
        for k, a in enumerate(c.axes):
            rec[f"{name}/axis{k}/data"] = a.data
            rec[f"{name}/axis{k}/x_coef"] = a.x_coef
            rec[f"{name}/axis{k}/y_coef"] = a.y_coef
        a0 = c.axes[0]
        rec[f"{name}/wbp0"] = oracle.ref_wbp(a0, v)
        # SIRT of axis 0 from its own WBP, with the per-iteration residual norms.
        s, n = oracle.ref_sirt(a0, v, rec[f"{name}/wbp0"], ni, ls)
        rec[f"{name}/sirt0"] = s
        rec[f"{name}/sirt0_norms"] = n
        rec[f"{name}/recon"] = oracle.ref_reconstruct(c.axes, v, no, ni, ls, rho)
        print(name, "done", flush=True)
    np.savez_compressed(out, **rec)
    print("wrote", out)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).with_name("ref_gpu.npz"))
