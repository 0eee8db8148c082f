"""End to end through the drop-in program: MRC mode-1 stacks and TXBR maps in
the reference's formats -> mtr_multiaxis -> MRC float32 volume, compared with
the oracle run on the same (int16-quantised) inputs."""
import subprocess

import numpy as np
import pytest

import cases
import mtr
import oracle
import phantom
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _write_inputs(tmp_path, case):
    """Quantise each stack to int16 (the reference reads mode 1 correctly only)."""
    sts, txbrs, qaxes = [], [], []
    for k, a in enumerate(case.axes):
        scale = 30000.0 / max(float(np.abs(a.data).max()), 1e-12)
        q = np.round(a.data * scale).astype(np.float32)
        st = tmp_path / f"axis{k}.st"
        mtr.write_mrc_stack(str(st), q, 1)
        tx = tmp_path / f"axis{k}.txbr"
        tx.write_text(phantom.txbr_text(a.x_coef, a.y_coef, case.vol))
        sts.append(str(st))
        txbrs.append(str(tx))
        qaxes.append(mtr.AxisData(a.x_coef, a.y_coef, q))
    return sts, txbrs, qaxes


@pytest.mark.parametrize("name,n,inner,rho,prec", [("two_axis", 2, 3, 0.8, "fp32"), ("single", 1, 10, 0.5, "fp32"),
                                                   ("mid", 1, 4, 0.7, "bf16")])
def test_cli_end_to_end(tmp_path, name, n, inner, rho, prec):
    c = cases.get(name)
    sts, txbrs, qaxes = _write_inputs(tmp_path, c)
    out = tmp_path / "out.mrc"
    cli = mtr.PKG / "bin" / "mtr_multiaxis"
    arg = f"{len(sts)}," + ",".join(sts + txbrs)
    r = subprocess.run([str(cli), "-i", arg, "-o", str(out), "-n", str(n), "-s", "0.5", "-m", str(rho), "--inner",
                        str(inner), "--precision", prec], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    h = mtr.read_mrc_header(str(out))
    v = c.vol
    assert (h.nx, h.ny, h.nz, h.mode) == (v.X, v.Y, v.Z, 2)
    assert (h.nxstart, h.nystart, h.nzstart) == (v.Xstart, v.Ystart, v.Zstart)
    got = mtr.read_mrc_stack(str(out))
    mode = oracle.REF_FAITHFUL if prec == "fp32" else oracle.FP64
    want = oracle.reconstruct(mode, qaxes, v, n, inner, 0.5, rho)
    assert rel_l2(got, want) < (1e-4 if prec == "fp32" else 1e-3)
    assert h.amin == pytest.approx(float(got.min())) and h.amax == pytest.approx(float(got.max()))


def test_cli_reports_missing_file(tmp_path):
    cli = mtr.PKG / "bin" / "mtr_multiaxis"
    r = subprocess.run([str(cli), "-i", f"1,{tmp_path}/none.st,{tmp_path}/none.txbr", "-o", str(tmp_path / "o.mrc")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "read MRC header" in r.stderr
