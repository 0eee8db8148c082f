"""ctypes binding of libmtr's C ABI (include/mtr.h).

This is a thin host-side mirror of the C entry points for tests, the
benchmark and Python callers.  It loads lib/libmtr.so built in-tree and
raises if the library is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path
from typing import Sequence

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libmtr.so"

OK = 0
STATUS = ["ok", "invalid argument", "CUDA error", "out of device memory", "I/O error", "format error",
          "unsupported", "no CUDA device", "timed out", "not ready", "over capacity"]
ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_OOM, ERR_IO, ERR_FORMAT, ERR_UNSUPPORTED, ERR_NO_DEVICE = 1, 2, 3, 4, 5, 6, 7
ERR_TIMEOUT, ERR_NOT_READY, ERR_CAPACITY = 8, 9, 10

PREC_FP32, PREC_MIXED_BF16, PREC_MIXED_FP16 = 0, 1, 2
MEM_HOST, MEM_DEVICE = 0, 1
FLAG_RECORD_NORMS, FLAG_GRAPH, FLAG_HOST_VOLUMES, FLAG_RECORD_CHANGES, FLAG_STREAM_SLABS = 1, 2, 4, 8, 16
MAX_AXES = 16
KERNEL_CLASSES = ["wbp", "forward", "residual", "backproject", "mace", "other"]
NOALLOC_SCRATCH_FLOATS = 8 * 1024 * 1024  # MTR_NOALLOC_SCRATCH_FLOATS


class MtrError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        name = STATUS[status] if 0 <= status < len(STATUS) else f"status {status}"
        super().__init__(f"{what}: {name}" if what else name)


class VolumeSize(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("Xstart", "Xend", "Ystart", "Yend", "Zstart", "Zend", "X", "Y", "Z")]

    @classmethod
    def make(cls, xs: int, xe: int, ys: int, ye: int, zs: int, ze: int) -> "VolumeSize":
        return cls(xs, xe, ys, ye, zs, ze, xe - xs, ye - ys, ze - zs)

    @property
    def shape(self) -> tuple[int, int, int]:
        """(Z, Y, X) numpy shape of a volume in this frame."""
        return (self.Z, self.Y, self.X)

    def astuple(self) -> tuple:
        return tuple(getattr(self, n) for n, _ in self._fields_)


class ProjectionSize(C.Structure):
    _fields_ = [("X", C.c_int), ("Y", C.c_int), ("AngN", C.c_int)]


class AxisC(C.Structure):
    _fields_ = [("prj", ProjectionSize), ("x_coef", C.POINTER(C.c_double)), ("y_coef", C.POINTER(C.c_double)),
                ("prj_data", C.c_void_p)]


class InstanceC(C.Structure):
    _fields_ = [("n_axes", C.c_int), ("axes", C.POINTER(AxisC)), ("vol", VolumeSize)]


class RequestC(C.Structure):
    _fields_ = [("n_axes", C.c_int), ("axes", C.POINTER(AxisC)), ("vol", VolumeSize), ("iter_times", C.c_int),
                ("sirt_inner", C.c_int), ("sirt_step", C.c_float), ("mace_step", C.c_float),
                ("out", C.POINTER(C.c_float))]


class XF(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("a11", "a12", "a21", "a22", "dx", "dy")]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("submitted", "completed", "queued", "active", "bytes_in_use",
                                             "peak_bytes", "budget_bytes", "steps", "voxel_updates")]


class Params(C.Structure):
    _fields_ = [("iter_times", C.c_int), ("sirt_inner", C.c_int), ("sirt_step", C.c_float),
                ("mace_step", C.c_float), ("precision", C.c_int), ("flags", C.c_int), ("slab_depth", C.c_int)]


class MrcHeader(C.Structure):
    _pack_ = 1
    _fields_ = ([(n, C.c_int) for n in ("nx", "ny", "nz", "mode", "nxstart", "nystart", "nzstart", "mx", "my", "mz")]
                + [(n, C.c_float) for n in ("xlen", "ylen", "zlen", "alpha", "beta", "gamma")]
                + [(n, C.c_int) for n in ("mapc", "mapr", "maps")]
                + [(n, C.c_float) for n in ("amin", "amax", "amean")]
                + [("ispg", C.c_short), ("nsymbt", C.c_short), ("next", C.c_int), ("creatid", C.c_short),
                   ("blank", C.c_char * 30), ("nint", C.c_short), ("nreal", C.c_short), ("sub", C.c_short),
                   ("zfac", C.c_short)]
                + [(n, C.c_float) for n in ("min2", "max2", "min3", "max3", "min4", "max4")]
                + [(n, C.c_short) for n in ("idtype", "lens", "nd1", "nd2", "vd1", "vd2")]
                + [("tiltangles", C.c_float * 6), ("xorg", C.c_float), ("yorg", C.c_float), ("zorg", C.c_float),
                   ("cmap", C.c_char * 4), ("stamp", C.c_char * 4), ("rms", C.c_float), ("nlabl", C.c_int),
                   ("labels", (C.c_char * 80) * 10)])


class OptionsC(C.Structure):
    _fields_ = [("number_tilt", C.c_int), ("mrc_path", (C.c_char * 1024) * MAX_AXES),
                ("txbr_path", (C.c_char * 1024) * MAX_AXES), ("out_path", C.c_char * 1024),
                ("block_x", C.c_int), ("block_y", C.c_int), ("block_z", C.c_int), ("iter_times", C.c_int),
                ("sirt_step", C.c_float), ("mace_step", C.c_float), ("sirt_inner", C.c_int),
                ("precision", C.c_int), ("help", C.c_int)]


_P = C.c_void_p
_SIGNATURES = {
    "mtr_abi_version": (C.c_int, []),
    "mtr_status_string": (C.c_char_p, [C.c_int]),
    "mtr_context_last_error": (C.c_char_p, [_P]),
    "mtr_params_default": (None, [C.POINTER(Params)]),
    "mtr_context_create": (C.c_int, [C.c_int, C.POINTER(_P)]),
    "mtr_context_destroy": (C.c_int, [_P]),
    "mtr_context_set_stream": (C.c_int, [_P, _P]),
    "mtr_context_synchronize": (C.c_int, [_P]),
    "mtr_context_trim": (C.c_int, [_P]),
    "mtr_context_launch_count": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "mtr_context_windowed_launch_count": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "mtr_set_wait_limit": (C.c_int, [C.c_longlong]),
    "mtr_context_set_profiling": (C.c_int, [_P, C.c_int]),
    "mtr_context_profile": (C.c_int, [_P, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
    "mtr_context_profile_reset": (C.c_int, [_P]),
    "mtr_wbp": (C.c_int, [_P, C.POINTER(AxisC), VolumeSize, C.c_int, C.c_int, _P]),
    "mtr_sirt": (C.c_int, [_P, C.POINTER(AxisC), VolumeSize, C.c_int, C.c_int, C.c_int, C.c_float, _P]),
    "mtr_sirt_noalloc": (C.c_int, [_P, ProjectionSize, _P, _P, _P, VolumeSize, C.c_int, C.c_int, C.c_int, C.c_float,
                                   _P]),
    "mtr_initial_z": (C.c_int, [_P, VolumeSize, _P, _P, _P]),
    "mtr_update_w": (C.c_int, [_P, VolumeSize, _P, _P, _P, C.c_float]),
    "mtr_reconstruct": (C.c_int, [_P, C.c_int, C.POINTER(AxisC), VolumeSize, C.POINTER(Params), _P]),
    "mtr_reconstruct_fp64": (C.c_int, [_P, C.c_int, C.POINTER(AxisC), VolumeSize, C.POINTER(Params), _P, C.c_int]),
    "mtr_recon_create": (C.c_int, [_P, C.c_int, C.POINTER(AxisC), VolumeSize, C.POINTER(Params), C.c_int,
                                   C.POINTER(_P)]),
    "mtr_recon_upload": (C.c_int, [_P, C.c_int, _P, C.c_int]),
    "mtr_recon_upload_half": (C.c_int, [_P, C.c_int, _P, C.c_int]),
    "mtr_recon_run": (C.c_int, [_P]),
    "mtr_recon_init": (C.c_int, [_P]),
    "mtr_recon_run_outer": (C.c_int, [_P, C.c_int, C.c_int]),
    "mtr_recon_save": (C.c_int, [_P, C.c_char_p]),
    "mtr_recon_load": (C.c_int, [_P, C.c_char_p, C.POINTER(C.c_int)]),
    "mtr_recon_download": (C.c_int, [_P, _P, C.c_int]),
    "mtr_recon_download_axes": (C.c_int, [_P, _P, C.c_int]),
    "mtr_recon_check": (C.c_int, [_P]),
    "mtr_recon_norms": (C.c_int, [_P, C.POINTER(C.c_double), C.c_longlong]),
    "mtr_recon_changes": (C.c_int, [_P, C.POINTER(C.c_double), C.c_int]),
    "mtr_recon_run_until": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(C.c_int)]),
    "mtr_recon_footprint": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "mtr_recon_describe": (C.c_int, [_P, C.c_char_p, C.c_int]),
    "mtr_recon_destroy": (C.c_int, [_P]),
    "mtr_estimate_footprint": (C.c_int, [C.c_int, C.POINTER(ProjectionSize), VolumeSize, C.c_int,
                                         C.POINTER(C.c_longlong)]),
    "mtr_batch_create": (C.c_int, [_P, C.c_int, C.POINTER(InstanceC), C.POINTER(Params), C.c_int, C.POINTER(_P)]),
    "mtr_batch_run": (C.c_int, [_P]),
    "mtr_batch_download": (C.c_int, [_P, C.c_int, _P, C.c_int]),
    "mtr_batch_info": (C.c_int, [_P, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "mtr_batch_destroy": (C.c_int, [_P]),
    "mtr_geometry_from_tilts": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(XF), C.c_double, C.c_int, C.c_int,
                                           VolumeSize, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mtr_tlt_read": (C.c_int, [C.c_char_p, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int)]),
    "mtr_txbr_write": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), VolumeSize]),
    "mtr_xf_read": (C.c_int, [C.c_char_p, C.POINTER(XF), C.c_int, C.POINTER(C.c_int)]),
    "mtr_server_create": (C.c_int, [_P, C.c_longlong, C.c_int, C.POINTER(_P)]),
    "mtr_server_submit": (C.c_int, [_P, C.POINTER(RequestC), C.POINTER(C.c_longlong)]),
    "mtr_server_step": (C.c_int, [_P, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_int)]),
    "mtr_server_stats_get": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "mtr_server_destroy": (C.c_int, [_P]),
    "mtr_mrc_read_header": (C.c_int, [C.c_char_p, C.POINTER(MrcHeader)]),
    "mtr_mrc_read_stack": (C.c_int, [C.c_char_p, _P, C.c_longlong]),
    "mtr_mrc_read_stack_device": (C.c_int, [_P, C.c_char_p, _P, C.c_longlong]),
    "mtr_mrc_read_stack_device_half": (C.c_int, [_P, C.c_char_p, _P, C.c_longlong]),
    "mtr_txbr_read": (C.c_int, [C.c_char_p, _P, _P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.POINTER(VolumeSize)]),
    "mtr_volume_size_empty": (None, [C.POINTER(VolumeSize)]),
    "mtr_mrc_write_volume": (C.c_int, [C.c_char_p, VolumeSize, _P]),
    "mtr_mrc_write_stack": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "mtr_parse_options": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), C.POINTER(OptionsC)]),
}

_lib: C.CDLL | None = None


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def load(path: str | Path | None = None) -> C.CDLL:
    """Load libmtr (build it first with __graft_entry__.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"libmtr not built: {p} is missing (run __graft_entry__.build())")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _ptr(a) -> int:
    """Address of a C-contiguous numpy array or a CUDA tensor."""
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        assert a.is_contiguous()
        return a.data_ptr()
    raise TypeError(f"unsupported buffer {type(a)}")


def _numel(a) -> int:
    return int(a.size) if isinstance(a, np.ndarray) else int(a.numel())


def _require_half(a, what: str) -> None:
    """FP16 entry points read 2 bytes per value: a buffer of any other type
    would be reinterpreted silently."""
    if isinstance(a, np.ndarray):
        ok = a.dtype == np.float16
    else:
        import torch

        ok = isinstance(a, torch.Tensor) and a.dtype == torch.float16
    if not ok:
        raise TypeError(f"{what}: needs IEEE FP16 data (numpy.float16 or torch.float16), got {getattr(a, 'dtype', type(a))}")


@dataclass
class AxisData:
    """One tilt axis: data [AngN, Y, X] float32 (numpy or CUDA tensor), coefficient arrays [AngN*4].
    `data` may instead be the shape tuple (AngN, Y, X) of an axis whose
    projections are uploaded after mtr_recon_create."""
    x_coef: np.ndarray
    y_coef: np.ndarray
    data: object

    def __post_init__(self):
        self.x_coef = np.ascontiguousarray(self.x_coef, dtype=np.float64).reshape(-1)
        self.y_coef = np.ascontiguousarray(self.y_coef, dtype=np.float64).reshape(-1)

    @property
    def prj(self) -> ProjectionSize:
        a, y, x = tuple(self.data) if isinstance(self.data, tuple) else tuple(self.data.shape)
        return ProjectionSize(x, y, a)

    def c_struct(self) -> AxisC:
        dp = C.POINTER(C.c_double)
        ptr = None if isinstance(self.data, tuple) else _ptr(self.data)
        return AxisC(self.prj, self.x_coef.ctypes.data_as(dp), self.y_coef.ctypes.data_as(dp), ptr)


def params(iter_times=5, sirt_inner=10, sirt_step=0.5, mace_step=0.7, precision=PREC_FP32, flags=0,
           slab_depth=0) -> Params:
    return Params(iter_times, sirt_inner, sirt_step, mace_step, precision, flags, slab_depth)


class Context:
    def __init__(self, device: int = 0):
        self.lib = load()
        h = _P()
        st = self.lib.mtr_context_create(device, C.byref(h))
        if st != OK:
            raise MtrError(st, "mtr_context_create")
        self.h = h

    def check(self, st: int, what: str) -> None:
        if st != OK:
            msg = self.lib.mtr_context_last_error(self.h)
            raise MtrError(st, f"{what} ({msg.decode() if msg else ''})")

    def close(self) -> None:
        if self.h:
            self.lib.mtr_context_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_ptr: int | None) -> None:
        self.check(self.lib.mtr_context_set_stream(self.h, stream_ptr or None), "set_stream")

    def trim(self) -> None:
        """Return the device memory the context's array pool holds in reserve."""
        self.check(self.lib.mtr_context_trim(self.h), "mtr_context_trim")

    def synchronize(self) -> None:
        self.check(self.lib.mtr_context_synchronize(self.h), "synchronize")

    def launch_count(self) -> int:
        n = C.c_longlong()
        self.check(self.lib.mtr_context_launch_count(self.h, C.byref(n)), "launch_count")
        return n.value

    def windowed_launch_count(self) -> int:
        """Launches of the TMA-windowed projector kernels issued so far."""
        n = C.c_longlong()
        self.check(self.lib.mtr_context_windowed_launch_count(self.h, C.byref(n)), "windowed_launch_count")
        return n.value

    def set_profiling(self, on: bool) -> None:
        self.check(self.lib.mtr_context_set_profiling(self.h, int(bool(on))), "set_profiling")

    def profile(self) -> dict:
        """{kernel class: (launches, total device ms)} since the last reset."""
        out = {}
        for k, name in enumerate(KERNEL_CLASSES):
            n, ms = C.c_longlong(), C.c_double()
            self.check(self.lib.mtr_context_profile(self.h, k, C.byref(n), C.byref(ms)), "profile")
            out[name] = (n.value, ms.value)
        return out

    def profile_reset(self) -> None:
        self.check(self.lib.mtr_context_profile_reset(self.h), "profile_reset")

    # --- reference-shaped entry points --------------------------------------------
    def wbp(self, axis: AxisData, vol: VolumeSize, z0: int | None = None, z1: int | None = None) -> np.ndarray:
        z0 = vol.Zstart if z0 is None else z0
        z1 = vol.Zend if z1 is None else z1
        out = np.zeros((z1 - z0, vol.Y, vol.X), np.float32)
        a = axis.c_struct()
        self.check(self.lib.mtr_wbp(self.h, C.byref(a), vol, z0, z1, _ptr(out)), "mtr_wbp")
        return out

    def sirt(self, axis: AxisData, vol: VolumeSize, slab: np.ndarray, n_inner=10, step=0.5, z0=None, z1=None):
        z0 = vol.Zstart if z0 is None else z0
        z1 = vol.Zend if z1 is None else z1
        out = np.ascontiguousarray(slab, dtype=np.float32).copy()
        a = axis.c_struct()
        self.check(self.lib.mtr_sirt(self.h, C.byref(a), vol, z0, z1, n_inner, step, _ptr(out)), "mtr_sirt")
        return out

    def initial_z(self, vol: VolumeSize, w: np.ndarray, wavg: np.ndarray) -> np.ndarray:
        z = np.empty(vol.shape, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        wavg = np.ascontiguousarray(wavg, np.float32)
        self.check(self.lib.mtr_initial_z(self.h, vol, _ptr(w), _ptr(wavg), _ptr(z)), "mtr_initial_z")
        return z

    def update_w(self, vol: VolumeSize, v: np.ndarray, z: np.ndarray, w: np.ndarray, step: float) -> np.ndarray:
        out = np.ascontiguousarray(w, np.float32).copy()
        v = np.ascontiguousarray(v, np.float32)
        z = np.ascontiguousarray(z, np.float32)
        self.check(self.lib.mtr_update_w(self.h, vol, _ptr(v), _ptr(z), _ptr(out), step), "mtr_update_w")
        return out

    def reconstruct(self, axes: Sequence[AxisData], vol: VolumeSize, p: Params) -> np.ndarray:
        arr = (AxisC * len(axes))(*[a.c_struct() for a in axes])
        out = np.empty(vol.shape, np.float32)
        self.check(self.lib.mtr_reconstruct(self.h, len(axes), arr, vol, C.byref(p), _ptr(out)), "mtr_reconstruct")
        return out


    def reconstruct_fp64(self, axes: Sequence[AxisData], vol: VolumeSize, p: Params, out=None,
                         mem_kind=MEM_HOST):
        """All-FP64 GPU reconstruction (error reference); returns float64 [Z, Y, X]."""
        arr = (AxisC * len(axes))(*[a.c_struct() for a in axes])
        if out is None:
            out = np.empty(vol.shape, np.float64)
        self.check(self.lib.mtr_reconstruct_fp64(self.h, len(axes), arr, vol, C.byref(p), _ptr(out), mem_kind),
                   "mtr_reconstruct_fp64")
        return out


class Recon:
    """Device-resident reconstruction (mtr_recon_*)."""

    def __init__(self, ctx: Context, axes: Sequence[AxisData], vol: VolumeSize, p: Params, mem_kind=MEM_HOST):
        self.ctx, self.vol, self.p, self.K = ctx, vol, p, len(axes)
        self._shapes = [(a.prj.AngN, a.prj.Y, a.prj.X) for a in axes]
        arr = (AxisC * len(axes))(*[a.c_struct() for a in axes])
        h = _P()
        ctx.check(ctx.lib.mtr_recon_create(ctx.h, len(axes), arr, vol, C.byref(p), mem_kind, C.byref(h)),
                  "mtr_recon_create")
        self.h = h

    def upload(self, k: int, data, mem_kind=MEM_HOST) -> None:
        self.ctx.check(self.ctx.lib.mtr_recon_upload(self.h, k, _ptr(data), mem_kind), "mtr_recon_upload")

    def upload_half(self, k: int, data, mem_kind=MEM_HOST) -> None:
        """Projections of axis k as IEEE FP16 (numpy float16 or a CUDA half tensor)."""
        _require_half(data, "upload_half")
        a, y, x = self._shapes[k]
        if _numel(data) != a * y * x:
            raise ValueError(f"upload_half: {_numel(data)} values given, axis {k} holds {a * y * x}")
        self.ctx.check(self.ctx.lib.mtr_recon_upload_half(self.h, k, _ptr(data), mem_kind), "mtr_recon_upload_half")

    def run(self) -> None:
        self.ctx.check(self.ctx.lib.mtr_recon_run(self.h), "mtr_recon_run")

    def download(self, out=None, mem_kind=MEM_HOST):
        if out is None:
            out = np.empty(self.vol.shape, np.float32)
        self.ctx.check(self.ctx.lib.mtr_recon_download(self.h, _ptr(out), mem_kind), "mtr_recon_download")
        return out

    def download_axes(self) -> np.ndarray:
        out = np.empty((self.K,) + self.vol.shape, np.float32)
        self.ctx.check(self.ctx.lib.mtr_recon_download_axes(self.h, _ptr(out), MEM_HOST), "download_axes")
        return out

    def norms(self) -> np.ndarray:
        n = self.p.iter_times * self.K * self.p.sirt_inner
        out = np.zeros(n, np.float64)
        self.ctx.check(self.ctx.lib.mtr_recon_norms(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), n), "norms")
        return out.reshape(self.p.iter_times, self.K, self.p.sirt_inner)

    def describe(self) -> list:
        """Kernels and tile shapes chosen per axis (JSON from mtr_recon_describe)."""
        import json

        buf = C.create_string_buffer(8192)
        self.ctx.check(self.ctx.lib.mtr_recon_describe(self.h, buf, len(buf)), "describe")
        return json.loads(buf.value.decode())

    def init(self) -> None:
        self.ctx.check(self.ctx.lib.mtr_recon_init(self.h), "mtr_recon_init")

    def run_outer(self, first: int, count: int) -> None:
        self.ctx.check(self.ctx.lib.mtr_recon_run_outer(self.h, first, count), "mtr_recon_run_outer")

    def save(self, path) -> None:
        self.ctx.check(self.ctx.lib.mtr_recon_save(self.h, str(path).encode()), "mtr_recon_save")

    def load(self, path) -> int:
        """Restore a checkpoint; returns the outer iterations it had done."""
        n = C.c_int()
        self.ctx.check(self.ctx.lib.mtr_recon_load(self.h, str(path).encode(), C.byref(n)), "mtr_recon_load")
        return n.value

    def changes(self, n: int) -> np.ndarray:
        """Relative L2 change of the consensus per outer iteration (FP64)."""
        out = np.zeros(n, np.float64)
        self.ctx.check(self.ctx.lib.mtr_recon_changes(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), n),
                       "mtr_recon_changes")
        return out

    def run_until(self, tol: float, first: int = 0) -> int:
        done = C.c_int()
        self.ctx.check(self.ctx.lib.mtr_recon_run_until(self.h, first, tol, C.byref(done)), "mtr_recon_run_until")
        return done.value

    def footprint(self) -> int:
        b = C.c_longlong()
        self.ctx.check(self.ctx.lib.mtr_recon_footprint(self.h, C.byref(b)), "footprint")
        return b.value

    def close(self) -> None:
        if self.h:
            self.ctx.lib.mtr_recon_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many reconstructions run together (mtr_batch_*): one persistent launch per
    SIRT phase over all instances, captured in a CUDA graph with FLAG_GRAPH."""

    def __init__(self, ctx: Context, instances: Sequence[tuple], p: Params, mem_kind=MEM_HOST):
        self.ctx, self.p = ctx, p
        self.vols = [vol for _, vol in instances]
        keep = []
        arr = (InstanceC * len(instances))()
        for i, (axes, vol) in enumerate(instances):
            ax = (AxisC * len(axes))(*[a.c_struct() for a in axes])
            keep.append(ax)
            arr[i] = InstanceC(len(axes), ax, vol)
        h = _P()
        ctx.check(ctx.lib.mtr_batch_create(ctx.h, len(instances), arr, C.byref(p), mem_kind, C.byref(h)),
                  "mtr_batch_create")
        self.h = h

    def run(self) -> None:
        self.ctx.check(self.ctx.lib.mtr_batch_run(self.h), "mtr_batch_run")

    def download(self, i: int, out=None, mem_kind=MEM_HOST):
        if out is None:
            out = np.empty(self.vols[i].shape, np.float32)
        self.ctx.check(self.ctx.lib.mtr_batch_download(self.h, i, _ptr(out), mem_kind), "mtr_batch_download")
        return out

    def info(self) -> dict:
        vu, by = C.c_longlong(), C.c_longlong()
        items = (C.c_longlong * 5)()
        self.ctx.check(self.ctx.lib.mtr_batch_info(self.h, C.byref(vu), C.byref(by), items), "mtr_batch_info")
        return {"voxel_updates": vu.value, "bytes": by.value,
                "items": dict(zip(["forward", "residual", "backproject", "mace", "own_launch_axes"], list(items)))}

    def close(self) -> None:
        if self.h:
            self.ctx.lib.mtr_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching server (mtr_server_*): requests are admitted by
    device footprint under `budget_bytes` and advance one SIRT iteration per
    step, all admitted requests in one persistent launch per phase."""

    def __init__(self, ctx: Context, budget_bytes: int, precision: int = PREC_FP32):
        self.ctx = ctx
        h = _P()
        ctx.check(ctx.lib.mtr_server_create(ctx.h, int(budget_bytes), precision, C.byref(h)), "mtr_server_create")
        self.h = h
        self._keep = {}  # id -> (axis structs, host arrays, output array)
        self._ids = (C.c_longlong * 4096)()

    def submit(self, axes: Sequence["AxisData"], vol: VolumeSize, iter_times: int, sirt_inner: int = 10,
               sirt_step: float = 0.5, mace_step: float = 0.7) -> int:
        if not all(isinstance(a.data, np.ndarray) for a in axes):
            raise TypeError("server requests take host (numpy) projections")
        out = np.empty(vol.shape, np.float32)
        ax = (AxisC * len(axes))(*[a.c_struct() for a in axes])
        req = RequestC(len(axes), ax, vol, iter_times, sirt_inner, sirt_step, mace_step,
                       out.ctypes.data_as(C.POINTER(C.c_float)))
        rid = C.c_longlong()
        self.ctx.check(self.ctx.lib.mtr_server_submit(self.h, C.byref(req), C.byref(rid)), "mtr_server_submit")
        self._keep[rid.value] = (ax, list(axes), out)
        return rid.value

    def step(self) -> list:
        """One scheduling step; returns [(id, volume)] of the requests retired."""
        n = C.c_int()
        self.ctx.check(self.ctx.lib.mtr_server_step(self.h, len(self._ids), self._ids, C.byref(n)), "mtr_server_step")
        return [(i, self._keep.pop(i)[2]) for i in self._ids[:n.value]]

    def stats(self) -> dict:
        st = ServerStats()
        self.ctx.check(self.ctx.lib.mtr_server_stats_get(self.h, C.byref(st)), "mtr_server_stats_get")
        return {n: getattr(st, n) for n, _ in ServerStats._fields_}

    def drain(self, max_steps: int = 1 << 30) -> dict:
        done = {}
        for _ in range(max_steps):
            for i, v in self.step():
                done[i] = v
            st = self.stats()
            if st["queued"] == 0 and st["active"] == 0:
                break
        return done

    def close(self) -> None:
        if self.h:
            self.ctx.lib.mtr_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --- file I/O --------------------------------------------------------------------------
def _check(st: int, what: str) -> None:
    if st != OK:
        raise MtrError(st, what)


def read_mrc_header(path: str) -> MrcHeader:
    h = MrcHeader()
    _check(load().mtr_mrc_read_header(str(path).encode(), C.byref(h)), "mtr_mrc_read_header")
    return h


def read_mrc_stack(path: str) -> np.ndarray:
    h = read_mrc_header(path)
    out = np.empty((h.nz, h.ny, h.nx), np.float32)
    _check(load().mtr_mrc_read_stack(str(path).encode(), _ptr(out), out.size), "mtr_mrc_read_stack")
    return out


def read_mrc_stack_device(ctx: "Context", path: str, out) -> None:
    """Read an MRC stack's data into a CUDA float32 tensor `out` (numel = nx*ny*nz)."""
    ctx.check(ctx.lib.mtr_mrc_read_stack_device(ctx.h, str(path).encode(), _ptr(out), out.numel()),
              "mtr_mrc_read_stack_device")


def read_mrc_stack_device_half(ctx: "Context", path: str, out, n: int | None = None) -> None:
    """Read an MRC stack's data into a CUDA float16 tensor `out`, rounded on the device.
    n: values to read (default nx*ny*nz of the file); `out` must hold exactly n halves."""
    _require_half(out, "read_mrc_stack_device_half")
    if n is None:
        h = read_mrc_header(path)
        n = h.nx * h.ny * h.nz
    if out.numel() != n:
        raise ValueError(f"read_mrc_stack_device_half: tensor holds {out.numel()} halves, {n} requested")
    ctx.check(ctx.lib.mtr_mrc_read_stack_device_half(ctx.h, str(path).encode(), _ptr(out), out.numel()),
              "mtr_mrc_read_stack_device_half")


def read_txbr(path: str, cap: int, vol: VolumeSize | None = None):
    lib = load()
    if vol is None:
        vol = VolumeSize()
        lib.mtr_volume_size_empty(C.byref(vol))
    x = np.zeros(cap, np.float64)
    y = np.zeros(cap, np.float64)
    nx, ny = C.c_int(), C.c_int()
    _check(lib.mtr_txbr_read(str(path).encode(), _ptr(x), _ptr(y), cap, C.byref(nx), C.byref(ny), C.byref(vol)),
           "mtr_txbr_read")
    return x[:nx.value], y[:ny.value], vol


def write_mrc_volume(path: str, vol: VolumeSize, data: np.ndarray) -> None:
    data = np.ascontiguousarray(data, np.float32)
    assert data.shape == vol.shape
    _check(load().mtr_mrc_write_volume(str(path).encode(), vol, _ptr(data)), "mtr_mrc_write_volume")


def write_mrc_stack(path: str, data: np.ndarray, mode: int = 1) -> None:
    data = np.ascontiguousarray(data, np.float32)
    nz, ny, nx = data.shape
    _check(load().mtr_mrc_write_stack(str(path).encode(), nx, ny, nz, mode, _ptr(data)), "mtr_mrc_write_stack")


def parse_options(argv: Sequence[str]) -> tuple[int, OptionsC]:
    args = [a.encode() for a in argv]
    arr = (C.c_char_p * (len(args) + 1))(*args, None)
    o = OptionsC()
    st = load().mtr_parse_options(len(args), arr, C.byref(o))
    return st, o


def geometry_from_tilts(tilt_deg, phi_deg: float, det_x: int, det_y: int, vol: VolumeSize,
                        xf=None) -> tuple[np.ndarray, np.ndarray]:
    """Per-view linear maps (x_coef, y_coef), [4*n] each, of a tilt series
    about an axis at in-plane angle phi; xf: optional [n, 6] alignment rows
    (a11 a12 a21 a22 dx dy) mapping raw view coordinates to aligned ones."""
    t = np.ascontiguousarray(tilt_deg, np.float64).reshape(-1)
    n = len(t)
    xs, ys = np.empty(4 * n), np.empty(4 * n)
    dp = C.POINTER(C.c_double)
    xfa = None
    if xf is not None:
        x = np.ascontiguousarray(xf, np.float64).reshape(n, 6)
        xfa = (XF * n)(*[XF(*row) for row in x])
    _check(load().mtr_geometry_from_tilts(n, t.ctypes.data_as(dp), xfa, float(phi_deg), det_x, det_y, vol,
                                          xs.ctypes.data_as(dp), ys.ctypes.data_as(dp)), "mtr_geometry_from_tilts")
    return xs, ys


def write_txbr(path: str, x_coef, y_coef, vol: VolumeSize) -> None:
    """TXBR file of the per-view maps (4 coefficients per view each) and vol's bounds."""
    x = np.ascontiguousarray(x_coef, np.float64).reshape(-1)
    y = np.ascontiguousarray(y_coef, np.float64).reshape(-1)
    if x.size != y.size or x.size % 4:
        raise ValueError("write_txbr: x and y maps need 4 coefficients per view each")
    dp = C.POINTER(C.c_double)
    _check(load().mtr_txbr_write(str(path).encode(), x.size // 4, x.ctypes.data_as(dp), y.ctypes.data_as(dp), vol),
           "mtr_txbr_write")


def read_tlt(path: str, cap: int = 100000) -> np.ndarray:
    out = np.empty(cap, np.float64)
    n = C.c_int()
    _check(load().mtr_tlt_read(str(path).encode(), out.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(n)),
           "mtr_tlt_read")
    return out[:n.value].copy()


def read_xf(path: str, cap: int = 100000) -> np.ndarray:
    arr = (XF * cap)()
    n = C.c_int()
    _check(load().mtr_xf_read(str(path).encode(), arr, cap, C.byref(n)), "mtr_xf_read")
    return np.array([[getattr(arr[i], f) for f, _ in XF._fields_] for i in range(n.value)], np.float64).reshape(-1, 6)


def estimate_footprint(prjs: Sequence[tuple[int, int, int]], vol: VolumeSize, precision: int) -> int:
    arr = (ProjectionSize * len(prjs))(*[ProjectionSize(*p) for p in prjs])
    b = C.c_longlong()
    _check(load().mtr_estimate_footprint(len(prjs), arr, vol, precision, C.byref(b)), "estimate_footprint")
    return b.value
