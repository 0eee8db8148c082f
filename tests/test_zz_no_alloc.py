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


def _noalloc_sirt(ctx, axis, vol, slab, n_inner, step):
    import torch

    lib = ctx.lib
    fn = lib.mtr_sirt_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, mtr.ProjectionSize, C.c_void_p, C.c_void_p, C.c_void_p, mtr.VolumeSize, C.c_int,
                   C.c_int, C.c_int, C.c_float, C.c_void_p]
    dev = torch.device("cuda", 0)
    xc = torch.from_numpy(np.ascontiguousarray(axis.x_coef)).to(dev)
    yc = torch.from_numpy(np.ascontiguousarray(axis.y_coef)).to(dev)
    b = torch.from_numpy(np.ascontiguousarray(axis.data, np.float32)).to(dev)
    x = torch.from_numpy(np.ascontiguousarray(slab, np.float32)).to(dev)
    torch.cuda.synchronize()
    st = fn(ctx.h, axis.prj, xc.data_ptr(), yc.data_ptr(), b.data_ptr(), vol, vol.Zstart, vol.Zend, n_inner, step,
            x.data_ptr())
    ctx.check(st, "mtr_sirt_noalloc")
    ctx.synchronize()
    return x.cpu().numpy()


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
