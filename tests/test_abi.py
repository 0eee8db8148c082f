"""The C-ABI library loads, exports every entry point include/mtr.h declares,
and behaves on a machine without a GPU (no compute calls are made here)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

import mtr

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(mtr_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("mtr_wbp", "mtr_sirt", "mtr_initial_z", "mtr_update_w", "mtr_reconstruct", "mtr_recon_create",
              "mtr_mrc_read_stack", "mtr_txbr_read", "mtr_mrc_write_volume", "mtr_parse_options"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(mtr.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_functions()) <= set(mtr.exported_symbols())


def test_abi_version_and_status_strings():
    lib = mtr.load()
    assert lib.mtr_abi_version() == 2
    assert lib.mtr_status_string(0) == b"ok"
    assert lib.mtr_status_string(3) == b"out of device memory"
    assert lib.mtr_status_string(999) == b"unknown status"


def test_params_default_matches_reference_options():
    # Options() defaults, ReadAndInitialOptions.h:33-42; inner count FunctionOnGPU.cu:212
    p = mtr.Params()
    mtr.load().mtr_params_default(ctypes.byref(p))
    assert (p.iter_times, p.sirt_inner, p.precision, p.flags) == (5, 10, 0, 0)
    assert p.sirt_step == pytest.approx(0.5) and p.mace_step == pytest.approx(0.7)


def test_null_arguments_rejected_without_device():
    lib = mtr.load()
    assert lib.mtr_context_create(0, None) == mtr.ERR_INVALID_ARGUMENT
    assert lib.mtr_recon_run(None) == mtr.ERR_INVALID_ARGUMENT
    assert lib.mtr_context_destroy(None) == 0
    assert lib.mtr_context_trim(None) == mtr.ERR_INVALID_ARGUMENT
    assert lib.mtr_recon_upload_half(None, 0, None, 0) == mtr.ERR_INVALID_ARGUMENT
    assert lib.mtr_mrc_read_stack_device_half(None, b"x.mrc", None, 1) == mtr.ERR_INVALID_ARGUMENT


def test_structs_match_c_layout():
    assert ctypes.sizeof(mtr.MrcHeader) == 1024
    assert ctypes.sizeof(mtr.VolumeSize) == 36
    assert ctypes.sizeof(mtr.ProjectionSize) == 12


def test_shape_only_axis_passes_null_data():
    """An axis given as a shape has no data pointer: mtr_recon_create then
    leaves its projections zero until an upload."""
    import numpy as np

    coef = np.zeros(4 * 3)
    a = mtr.AxisData(coef, coef, (3, 5, 7)).c_struct()
    assert (a.prj.X, a.prj.Y, a.prj.AngN) == (7, 5, 3)
    assert not a.prj_data
    b = mtr.AxisData(coef, coef, np.zeros((3, 5, 7), np.float32)).c_struct()
    assert b.prj_data


def test_no_device_reports_status():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = mtr.load().mtr_context_create(0, ctypes.byref(h))
    assert st == mtr.ERR_NO_DEVICE


def test_cli_help_and_bad_options():
    cli = mtr.PKG / "bin" / "mtr_multiaxis"
    r = subprocess.run([str(cli), "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "-i K" in r.stdout
    r = subprocess.run([str(cli), "-q"], capture_output=True, text=True)
    assert r.returncode != 0
    r = subprocess.run([str(cli), "-i", "2,a.st,a.txbr", "-o", "x.mrc"], capture_output=True, text=True)
    assert r.returncode != 0  # K=2 needs 4 paths


def test_half_entry_points_reject_other_dtypes():
    """The FP16 upload and reader read 2 bytes per value: any other dtype is
    refused before the library sees it."""
    import numpy as np

    with pytest.raises(TypeError):
        mtr._require_half(np.zeros(4, np.float32), "upload_half")
    with pytest.raises(TypeError):
        mtr._require_half(np.zeros(4, np.uint16), "upload_half")
    mtr._require_half(np.zeros(4, np.float16), "upload_half")
