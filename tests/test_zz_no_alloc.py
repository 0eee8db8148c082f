"""mtr_sirt_noalloc: SIRT for callers that cannot allocate device memory where
they reconstruct (a pipeline stage that must not synchronise the device, a
program whose device memory belongs to another allocator).  Called through
the C ABI with device buffers the caller owns; its output must match the
allocating entry point mtr_sirt, on two calls in a row (the fixed scratch is
shared between calls and must be cleared by each).

This file sorts last so that a run stopping at the first failure has already
run every other test."""
import ctypes as C

import numpy as np
import pytest

import cases
import mtr
from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5  # same kernels as mtr_sirt; float atomics add in an unspecified order


def _noalloc_status(ctx, axis, vol, slab, n_inner, step, z0=None, z1=None):
    """Calls mtr_sirt_noalloc on device copies of the inputs; returns (status, slab)."""
    import torch

    lib = ctx.lib
    fn = lib.mtr_sirt_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, mtr.ProjectionSize, C.c_void_p, C.c_void_p, C.c_void_p, mtr.VolumeSize, C.c_int,
                   C.c_int, C.c_int, C.c_float, C.c_void_p]
    z0 = vol.Zstart if z0 is None else z0
    z1 = vol.Zend if z1 is None else z1
    dev = torch.device("cuda", 0)
    xc = torch.from_numpy(np.ascontiguousarray(axis.x_coef)).to(dev)
    yc = torch.from_numpy(np.ascontiguousarray(axis.y_coef)).to(dev)
    b = torch.from_numpy(np.ascontiguousarray(axis.data, np.float32)).to(dev)
    x = torch.from_numpy(np.ascontiguousarray(slab, np.float32)).to(dev)
    torch.cuda.synchronize()
    st = fn(ctx.h, axis.prj, xc.data_ptr(), yc.data_ptr(), b.data_ptr(), vol, z0, z1, n_inner, step, x.data_ptr())
    ctx.synchronize()
    return st, x.cpu().numpy()


def _noalloc_sirt(ctx, axis, vol, slab, n_inner, step, z0=None, z1=None):
    st, out = _noalloc_status(ctx, axis, vol, slab, n_inner, step, z0, z1)
    ctx.check(st, "mtr_sirt_noalloc")
    return out


@pytest.fixture(scope="module")
def nctx():
    c = mtr.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", ["single", "rect"])
def test_noalloc_matches_allocating_entry_point_twice(nctx, name):
    c = cases.get(name)
    a = c.axes[0]
    x0 = nctx.wbp(a, c.vol)
    want = nctx.sirt(a, c.vol, x0, n_inner=5, step=0.5)
    first = _noalloc_sirt(nctx, a, c.vol, x0, 5, 0.5)
    second = _noalloc_sirt(nctx, a, c.vol, x0, 5, 0.5)
    assert rel_l2(first, want) < TOL
    assert rel_l2(second, want) < TOL


def test_noalloc_rejects_sizes_beyond_its_scratch(nctx):
    import torch

    fn = nctx.lib.mtr_sirt_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, mtr.ProjectionSize, C.c_void_p, C.c_void_p, C.c_void_p, mtr.VolumeSize, C.c_int,
                   C.c_int, C.c_int, C.c_float, C.c_void_p]
    dummy = torch.zeros(16, device="cuda")
    prj = mtr.ProjectionSize(2048, 2048, 61)  # 3 * 2048^2 * 61 floats > the fixed scratch
    vol = mtr.VolumeSize.make(0, 8, 0, 8, 0, 8)
    st = fn(nctx.h, prj, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), vol, 0, 8, 1, 0.5, dummy.data_ptr())
    assert st == mtr.ERR_CAPACITY
    assert b"exceeds the fixed scratch" in nctx.lib.mtr_context_last_error(nctx.h)


def test_noalloc_slab_offset_matches_allocating_entry_point(nctx):
    """A Z-slab that does not start at the volume's first plane (the slab
    origin moves the volume index base of every kernel)."""
    c = cases.get("single")
    a, v = c.axes[0], c.vol
    z0, z1 = v.Zstart + 3, v.Zstart + 7
    x0 = nctx.wbp(a, v, z0, z1)
    want = nctx.sirt(a, v, x0, n_inner=4, step=0.5, z0=z0, z1=z1)
    got = _noalloc_sirt(nctx, a, v, x0, 4, 0.5, z0, z1)
    assert rel_l2(got, want) < TOL


def _sized_case(depth: int):
    """64x64 detector with 600 tilts and a 64x64xdepth volume: 3*600*64*64 +
    64*64*depth floats of scratch, exactly the fixed array at depth 248."""
    import phantom

    vol = mtr.VolumeSize.make(0, 64, 0, 64, 0, depth)
    xc, yc = phantom.axis_maps(64, 64, np.linspace(-60.0, 60.0, 600), 0.0, vol)
    rng = np.random.default_rng(7)
    data = rng.uniform(0.0, 1.0, (600, 64, 64)).astype(np.float32)
    return mtr.AxisData(xc, yc, data), vol


def test_noalloc_accepts_exactly_its_capacity_and_rejects_one_plane_more(nctx):
    a, v = _sized_case(248)
    assert 3 * 600 * 64 * 64 + 64 * 64 * 248 == mtr.NOALLOC_SCRATCH_FLOATS
    x0 = nctx.wbp(a, v)
    want = nctx.sirt(a, v, x0, n_inner=1, step=0.5)
    st, got = _noalloc_status(nctx, a, v, x0, 1, 0.5)
    assert st == mtr.OK
    assert rel_l2(got, want) < TOL
    a2, v2 = _sized_case(249)
    st, _ = _noalloc_status(nctx, a2, v2, np.zeros(v2.shape, np.float32), 1, 0.5)
    assert st == mtr.ERR_CAPACITY
