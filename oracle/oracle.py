"""ctypes binding of the CPU oracle (oracle.cpp) and of the harness that runs
the reference's own kernels (ref_runner.cu).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the oracle results are compared
with, never as the product.

mode 0 = reference-faithful precision, mode 1 = all FP64 (see oracle.cpp).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Sequence

import numpy as np

ORACLE = Path(__file__).resolve().parent
LIB = ORACLE / "liboracle.so"
REFRUN = ORACLE / "liborc_refrun.so"
REF_CUBIN = ORACLE / "_ref" / "ref_kernels.cubin"

REF_FAITHFUL, FP64 = 0, 1


class OrcVol(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("Xstart", "Xend", "Ystart", "Yend", "Zstart", "Zend", "X", "Y", "Z")]


class OrcPrj(C.Structure):
    _fields_ = [("X", C.c_int), ("Y", C.c_int), ("AngN", C.c_int)]


_P = C.c_void_p
_lib = None
_rr = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise FileNotFoundError(f"oracle not built: {LIB} (run oracle/build.py)")
        _lib = C.CDLL(str(LIB))
        _lib.orc_wbp.argtypes = [C.c_int, OrcPrj, OrcVol, _P, _P, _P, C.c_int, C.c_int, _P]
        _lib.orc_forward.argtypes = [C.c_int, OrcPrj, OrcVol, _P, _P, _P, C.c_int, C.c_int, _P, _P]
        _lib.orc_backproject.argtypes = [OrcPrj, OrcVol, _P, _P, _P, C.c_int, C.c_int, _P, _P]
        _lib.orc_sirt.argtypes = [C.c_int, OrcPrj, OrcVol, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_double, _P, _P]
        _lib.orc_reconstruct.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, OrcVol, C.c_int, C.c_int, C.c_double,
                                         C.c_double, _P, _P, _P]
        _lib.orc_divide_slice.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _lib.orc_set_threads.argtypes = [C.c_int]
        _lib.orc_num_threads.restype = C.c_int
    return _lib


def _vol(vol) -> OrcVol:
    return OrcVol(*[int(getattr(vol, n)) for n, _ in OrcVol._fields_])


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def set_threads(n: int) -> None:
    load().orc_set_threads(int(n))


def num_threads() -> int:
    return load().orc_num_threads()


def divide_slice(myid: int, n: int, z: int, s: int) -> tuple[int, int]:
    a, b = C.c_int(), C.c_int()
    load().orc_divide_slice(myid, n, z, s, C.byref(a), C.byref(b))
    return a.value, b.value


def wbp(mode: int, axis, vol, z0=None, z1=None) -> np.ndarray:
    z0 = vol.Zstart if z0 is None else z0
    z1 = vol.Zend if z1 is None else z1
    d = _f32(axis.data)
    a, y, x = d.shape
    xc, yc = _f64(axis.x_coef), _f64(axis.y_coef)
    out = np.zeros((z1 - z0, vol.Y, vol.X), np.float64)
    load().orc_wbp(mode, OrcPrj(x, y, a), _vol(vol), xc.ctypes.data, yc.ctypes.data, d.ctypes.data, z0, z1,
                   out.ctypes.data)
    return out


def forward(mode: int, axis, vol, slab, z0=None, z1=None):
    z0 = vol.Zstart if z0 is None else z0
    z1 = vol.Zend if z1 is None else z1
    a, y, x = axis.data.shape
    xc, yc = _f64(axis.x_coef), _f64(axis.y_coef)
    sl = _f64(slab)
    s = np.zeros((a, y, x), np.float64)
    c = np.zeros((a, y, x), np.float64)
    load().orc_forward(mode, OrcPrj(x, y, a), _vol(vol), xc.ctypes.data, yc.ctypes.data, sl.ctypes.data, z0, z1,
                       s.ctypes.data, c.ctypes.data)
    return s, c


def backproject(axis, vol, r, z0=None, z1=None):
    z0 = vol.Zstart if z0 is None else z0
    z1 = vol.Zend if z1 is None else z1
    a, y, x = axis.data.shape
    xc, yc = _f64(axis.x_coef), _f64(axis.y_coef)
    rr = _f64(r)
    s = np.zeros((z1 - z0, vol.Y, vol.X), np.float64)
    c = np.zeros_like(s)
    load().orc_backproject(OrcPrj(x, y, a), _vol(vol), xc.ctypes.data, yc.ctypes.data, rr.ctypes.data, z0, z1,
                           s.ctypes.data, c.ctypes.data)
    return s, c


def sirt(mode: int, axis, vol, slab, n_inner=10, step=0.5, z0=None, z1=None, norms=False):
    z0 = vol.Zstart if z0 is None else z0
    z1 = vol.Zend if z1 is None else z1
    d = _f32(axis.data)
    a, y, x = d.shape
    xc, yc = _f64(axis.x_coef), _f64(axis.y_coef)
    out = _f64(slab).copy()
    nrm = np.zeros(max(1, n_inner), np.float64)
    load().orc_sirt(mode, OrcPrj(x, y, a), _vol(vol), xc.ctypes.data, yc.ctypes.data, d.ctypes.data, z0, z1,
                    n_inner, step, out.ctypes.data, nrm.ctypes.data)
    return (out, nrm[:n_inner]) if norms else out


def reconstruct(mode: int, axes: Sequence, vol, n_outer=5, n_inner=10, sirt_step=0.5, mace_step=0.7,
                with_axes=False, with_norms=False):
    K = len(axes)
    datas = [_f32(a.data) for a in axes]
    xcs = [_f64(a.x_coef) for a in axes]
    ycs = [_f64(a.y_coef) for a in axes]
    prjs = (OrcPrj * K)(*[OrcPrj(d.shape[2], d.shape[1], d.shape[0]) for d in datas])
    pd = (C.c_void_p * K)(*[d.ctypes.data for d in datas])
    px = (C.c_void_p * K)(*[x.ctypes.data for x in xcs])
    py = (C.c_void_p * K)(*[y.ctypes.data for y in ycs])
    out = np.zeros((vol.Z, vol.Y, vol.X), np.float64)
    ow = np.zeros((K, vol.Z, vol.Y, vol.X), np.float64) if with_axes else None
    nr = np.zeros((max(1, n_outer), K, max(1, n_inner)), np.float64) if with_norms else None
    load().orc_reconstruct(mode, K, C.addressof(prjs), C.addressof(px), C.addressof(py), C.addressof(pd), _vol(vol),
                           n_outer, n_inner, sirt_step, mace_step, out.ctypes.data,
                           ow.ctypes.data if ow is not None else None, nr.ctypes.data if nr is not None else None)
    res = [out]
    if with_axes:
        res.append(ow)
    if with_norms:
        res.append(nr)
    return res[0] if len(res) == 1 else tuple(res)


# --- the reference's own kernels, from the cubin built out of FunctionOnGPU.cu ----------
def refrun_available() -> bool:
    return REFRUN.exists() and REF_CUBIN.exists()


def _refrun() -> C.CDLL:
    global _rr
    if _rr is None:
        if not refrun_available():
            raise FileNotFoundError("reference kernels not available (oracle/_ref/ref_kernels.cubin)")
        _rr = C.CDLL(str(REFRUN))
        _rr.rr_last_error.restype = C.c_char_p
        _rr.rr_load.argtypes = [C.c_char_p]
        _rr.rr_wbp.argtypes = [_P, _P, _P, _P, _P, C.c_int, C.c_int, _P]
        _rr.rr_sirt.argtypes = [_P, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_float, _P, _P]
        _rr.rr_reconstruct.argtypes = [C.c_int, _P, _P, _P, _P, _P, C.c_int, C.c_int, C.c_float, C.c_float, _P]
        if _rr.rr_load(str(REF_CUBIN).encode()) != 0:
            raise RuntimeError("rr_load: " + _rr.rr_last_error().decode())
    return _rr


def _rr_check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what}: {_refrun().rr_last_error().decode()}")


def ref_wbp(axis, vol, z0=None, z1=None) -> np.ndarray:
    rr = _refrun()
    z0 = vol.Zstart if z0 is None else z0
    z1 = vol.Zend if z1 is None else z1
    d = _f32(axis.data)
    prj = np.array([d.shape[2], d.shape[1], d.shape[0]], np.int32)
    v = np.array([getattr(vol, n) for n, _ in OrcVol._fields_], np.int32)
    xc, yc = _f64(axis.x_coef), _f64(axis.y_coef)
    out = np.zeros((z1 - z0, vol.Y, vol.X), np.float32)
    _rr_check(rr.rr_wbp(prj.ctypes.data, v.ctypes.data, xc.ctypes.data, yc.ctypes.data, d.ctypes.data, z0, z1,
                        out.ctypes.data), "rr_wbp")
    return out


def ref_sirt(axis, vol, slab, n_inner=10, step=0.5, z0=None, z1=None):
    rr = _refrun()
    z0 = vol.Zstart if z0 is None else z0
    z1 = vol.Zend if z1 is None else z1
    d = _f32(axis.data)
    prj = np.array([d.shape[2], d.shape[1], d.shape[0]], np.int32)
    v = np.array([getattr(vol, n) for n, _ in OrcVol._fields_], np.int32)
    xc, yc = _f64(axis.x_coef), _f64(axis.y_coef)
    out = _f32(slab).copy()
    nrm = np.zeros(max(1, n_inner), np.float64)
    _rr_check(rr.rr_sirt(prj.ctypes.data, v.ctypes.data, xc.ctypes.data, yc.ctypes.data, d.ctypes.data, z0, z1,
                         n_inner, step, out.ctypes.data, nrm.ctypes.data), "rr_sirt")
    return out, nrm[:n_inner]


def ref_reconstruct(axes: Sequence, vol, n_outer=5, n_inner=10, sirt_step=0.5, mace_step=0.7) -> np.ndarray:
    rr = _refrun()
    K = len(axes)
    datas = [_f32(a.data) for a in axes]
    xcs = [_f64(a.x_coef) for a in axes]
    ycs = [_f64(a.y_coef) for a in axes]
    prj = np.array([[d.shape[2], d.shape[1], d.shape[0]] for d in datas], np.int32).reshape(-1)
    v = np.array([getattr(vol, n) for n, _ in OrcVol._fields_], np.int32)
    pd = (C.c_void_p * K)(*[d.ctypes.data for d in datas])
    px = (C.c_void_p * K)(*[x.ctypes.data for x in xcs])
    py = (C.c_void_p * K)(*[y.ctypes.data for y in ycs])
    out = np.zeros((vol.Z, vol.Y, vol.X), np.float32)
    _rr_check(rr.rr_reconstruct(K, prj.ctypes.data, C.addressof(px), C.addressof(py), C.addressof(pd), v.ctypes.data,
                                n_outer, n_inner, sirt_step, mace_step, out.ctypes.data), "rr_reconstruct")
    return out
