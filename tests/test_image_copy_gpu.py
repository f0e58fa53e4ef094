"""GPU: image memory through the C ABI -- hgb_image_create / write / read and
the device-to-device copies hgb_image_copy and hgb_image_copy_region, which
replace hipaccCopyMemory and hipaccCopyMemoryRegion
(runtime/hipacc_cu_standalone.hpp:165-216).  Every copy is checked against
numpy slicing of the same host arrays, for several storage types, pitches
(alignments) and windows, including windows on the image edges and 1-pixel
windows; bad windows and mismatched images are rejected on the host.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (hgb dtype, numpy dtype, channels)
TYPES = [(0, np.uint8, 1), (1, np.uint8, 4), (2, np.int16, 1), (9, np.float32, 1), (8, np.uint16, 1),
         (10, np.float64, 1)]


def _rand(rng, npdt, h, w, ch):
    shape = (h, w) if ch == 1 else (h, w, ch)
    if npdt == np.float32 or npdt == np.float64:
        return rng.random(shape).astype(npdt)
    info = np.iinfo(npdt)
    return rng.integers(info.min, info.max, shape, endpoint=True, dtype=npdt)


class Img:
    def __init__(self, lib, dt, w, h, align, host=None):
        self.lib = lib
        self.p = C.c_void_p()
        rc = lib.hgb_image_create(dt, w, h, align, None if host is None else host.ctypes.data_as(C.c_void_p),
                                  C.byref(self.p))
        assert rc == 0
        self.w, self.h = w, h

    def read(self, like):
        out = np.empty_like(like)
        assert self.lib.hgb_image_read(self.p, out.ctypes.data_as(C.c_void_p), None) == 0
        return out

    def write(self, a):
        assert self.lib.hgb_image_write(self.p, np.ascontiguousarray(a).ctypes.data_as(C.c_void_p), None) == 0

    def close(self):
        self.lib.hgb_image_destroy(self.p)


@pytest.mark.parametrize("dt,npdt,ch", TYPES)
@pytest.mark.parametrize("align", [0, 64, 512])
def test_copy_whole_image(gpu, dt, npdt, ch, align):
    from hipacc_gb300 import _lib as L

    lib = L.load()
    rng = np.random.default_rng(dt * 7 + align)
    w, h = 333, 77
    a = _rand(rng, npdt, h, w, ch)
    src = Img(lib, dt, w, h, align, a)
    dst = Img(lib, dt, w, h, 256)
    assert lib.hgb_image_copy(src.p, dst.p, None) == 0
    assert np.array_equal(dst.read(a), a)
    # overwrite the source: the copy is a separate buffer
    b = _rand(rng, npdt, h, w, ch)
    src.write(b)
    assert np.array_equal(dst.read(a), a) and np.array_equal(src.read(b), b)
    src.close()
    dst.close()


@pytest.mark.parametrize("dt,npdt,ch", TYPES)
def test_copy_region_windows(gpu, dt, npdt, ch):
    from hipacc_gb300 import _lib as L

    lib = L.load()
    rng = np.random.default_rng(100 + dt)
    sw, sh, dw, dh = 257, 131, 190, 203
    a = _rand(rng, npdt, sh, sw, ch)
    d0 = _rand(rng, npdt, dh, dw, ch)
    src = Img(lib, dt, sw, sh, 0, a)
    dst = Img(lib, dt, dw, dh, 128, d0)
    expect = d0.copy()
    # (src window, dst window): interior, edges, corners, single pixels, full rows
    cases = [((10, 20, 50, 40), (3, 7, 50, 40)), ((0, 0, 1, 1), (dw - 1, dh - 1, 1, 1)),
             ((sw - 64, sh - 9, 64, 9), (0, 0, 64, 9)), ((0, 5, sw - 100, 1), (0, dh - 1, sw - 100, 1)),
             ((100, 0, 1, sh), (dw - 1, 0, 1, sh)), ((31, 17, 190, 100), (0, 103, 190, 100))]
    for sw_, dw_ in cases:
        rc = lib.hgb_image_copy_region(src.p, C.byref(L.Window(*sw_)), dst.p, C.byref(L.Window(*dw_)), None)
        assert rc == 0, L.load().hgb_last_error()
        sx, sy, ww, hh = sw_
        dx, dy, _, _ = dw_
        expect[dy:dy + hh, dx:dx + ww] = a[sy:sy + hh, sx:sx + ww]
        assert np.array_equal(dst.read(d0), expect), (sw_, dw_)
    src.close()
    dst.close()


def test_copy_region_null_windows_and_errors(gpu):
    from hipacc_gb300 import _lib as L

    lib = L.load()
    rng = np.random.default_rng(3)
    a = rng.random((40, 60)).astype(np.float32)
    src = Img(lib, 9, 60, 40, 0, a)
    dst = Img(lib, 9, 60, 40, 0)
    # NULL windows: the whole images (same size)
    assert lib.hgb_image_copy_region(src.p, None, dst.p, None, None) == 0
    assert np.array_equal(dst.read(a), a)
    small = Img(lib, 9, 30, 40, 0)
    u8 = Img(lib, 0, 60, 40, 0)
    # window past the edge, negative offset, different window sizes, dtype or size mismatch
    bad = [(src.p, L.Window(50, 0, 11, 10), dst.p, L.Window(0, 0, 11, 10)),
           (src.p, L.Window(-1, 0, 10, 10), dst.p, L.Window(0, 0, 10, 10)),
           (src.p, L.Window(0, 0, 10, 10), dst.p, L.Window(0, 0, 10, 11)),
           (src.p, L.Window(0, 0, 10, 10), u8.p, L.Window(0, 0, 10, 10))]
    for s, sw_, d, dw_ in bad:
        assert lib.hgb_image_copy_region(s, C.byref(sw_), d, C.byref(dw_), None) == L.ERR_INVALID
    assert lib.hgb_image_copy(src.p, small.p, None) == L.ERR_INVALID
    assert lib.hgb_image_copy(src.p, u8.p, None) == L.ERR_INVALID
    assert lib.hgb_image_copy(None, dst.p, None) == L.ERR_INVALID
    for im in (src, dst, small, u8):
        im.close()


def test_copy_on_stream_orders_with_kernels(gpu):
    """A copy queued on a stream after a kernel sees the kernel's result."""
    import torch

    from hipacc_gb300 import _lib as L

    lib = L.load()
    rng = np.random.default_rng(9)
    a = rng.integers(0, 256, (96, 128, 4), dtype=np.uint8)
    rgba = Img(lib, 1, 128, 96, 0, a)
    gray = Img(lib, 0, 128, 96, 0)
    copy = Img(lib, 0, 128, 96, 0)
    s = torch.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    vi, vo = L.View(), L.View()
    L.check(lib.hgb_image_get_view(rgba.p, C.byref(vi)))
    L.check(lib.hgb_image_get_view(gray.p, C.byref(vo)))
    L.check(lib.hgb_point_gray(C.byref(vi), C.byref(vo), 77, 150, 29, 8, sp))
    L.check(lib.hgb_image_copy_region(gray.p, C.byref(L.Window(8, 4, 100, 80)), copy.p,
                                      C.byref(L.Window(0, 0, 100, 80)), sp))
    s.synchronize()
    a32 = a.astype(np.uint32)
    g = ((77 * a32[..., 0] + 150 * a32[..., 1] + 29 * a32[..., 2]) >> 8).astype(np.uint8)
    got = copy.read(np.zeros((96, 128), np.uint8))
    assert np.array_equal(got[:80, :100], g[4:84, 8:108])
    for im in (rgba, gray, copy):
        im.close()
