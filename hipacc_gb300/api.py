"""Python front end of the C ABI for torch CUDA tensors.

Images are tensors of shape (H, W) or (B, H, W); RGBA images are uint8
tensors of shape (H, W, 4) or (B, H, W, 4).  Every call goes through
libhipacc_gb300.so on the tensor's device and current stream; nothing here
computes pixels itself.
"""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np
import torch

from . import _lib as L
from ._lib import CLAMP, CONSTANT, MAX, MIN, MIRROR, PROD, REPEAT, SUM, UNDEFINED  # noqa: F401

_DT = {torch.uint8: L.U8, torch.int16: L.I16, torch.int32: L.I32, torch.float16: L.F16,
       torch.bfloat16: L.BF16, torch.float32: L.F32, torch.float64: L.F64, torch.int64: L.U64}

SOBEL3_X = np.array([[-1, 0, 1], [-2, 0, 2], [-1, 0, 1]], np.int32)
SOBEL3_Y = np.array([[-1, -2, -1], [0, 0, 0], [1, 2, 1]], np.int32)


def view(t: torch.Tensor, rgba: bool = False) -> L.View:
    """hgb_view of a CUDA tensor (rows may be padded; the last dim must be dense)."""
    if not t.is_cuda:
        raise ValueError("hipacc_gb300 operates on CUDA tensors")
    es = t.element_size()
    if rgba:
        if t.dtype != torch.uint8 or t.shape[-1] != 4 or t.stride(-1) != 1 or t.stride(-2) != 4:
            raise ValueError("RGBA images are uint8 tensors (..., H, W, 4) with dense pixels")
        shape = t.shape[:-1]
        strides = t.stride()[:-1]
        dt = L.U8X4
    else:
        if t.stride(-1) != 1:
            raise ValueError("the innermost dimension must be dense")
        shape, strides, dt = t.shape, t.stride(), _DT[t.dtype]
    if len(shape) == 2:
        b, (h, w) = 1, shape
        bs = strides[0] * es * h
    elif len(shape) == 3:
        b, h, w = shape
        bs = strides[0] * es
    else:
        raise ValueError("images are (H, W) or (B, H, W)")
    pitch = strides[-2] * es
    return L.View(t.data_ptr(), dt, int(w), int(h), int(b), int(pitch), int(bs))


def window(w):
    if w is None:
        return None
    return C.byref(L.Window(*[int(v) for v in w]))


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _fptr(a):
    if a is None:
        return None
    a = np.ascontiguousarray(a, np.float32)
    return a.ctypes.data_as(C.c_void_p), a


def init(device: int = 0) -> str:
    buf = C.create_string_buffer(256)
    L.call("hgb_init", device, buf, 256)
    return buf.value.decode()


def local_op(inp, out=None, mask=None, domain=None, size=None, reduce=SUM, boundary=CLAMP, const=0.0, acc=None,
             iter_space=None, mask_dev=None, stream=None):
    """Kernel::convolve / reduce(Domain) as one launch (hgb_local_op)."""
    if out is None:
        out = torch.empty_like(inp)
    if mask is not None:
        m = np.ascontiguousarray(mask, np.float32)
        mh, mw = m.shape
    elif mask_dev is not None:
        mh, mw = size
        m = None
    else:
        mh, mw = size if size is not None else np.asarray(domain).shape
        m = None
    d = None if domain is None else np.ascontiguousarray(domain, np.uint8)
    vi, vo = view(inp), view(out)
    L.call("hgb_local_op", C.byref(vi), window(acc), C.byref(vo), window(iter_space),
           None if m is None else m.ctypes.data_as(C.c_void_p),
           None if mask_dev is None else C.c_void_p(mask_dev.data_ptr()),
           None if d is None else d.ctypes.data_as(C.c_void_p), mw, mh, reduce, boundary, float(const),
           _stream(stream))
    return out


def sobel_mag(inp, out=None, mask_x=SOBEL3_X, mask_y=SOBEL3_Y, boundary=MIRROR, const=0, sum_out=None, max_out=None,
              stream=None):
    """Sobel magnitude with fused u64 sum / u8 max (device tensors of 1 int64 / int32)."""
    if out is None:
        out = torch.empty_like(inp)
    mx = np.ascontiguousarray(mask_x, np.int32)
    my = np.ascontiguousarray(mask_y, np.int32)
    vi, vo = view(inp), view(out)
    L.call("hgb_sobel_mag", C.byref(vi), C.byref(vo), mx.ctypes.data_as(C.c_void_p), my.ctypes.data_as(C.c_void_p),
           mx.shape[0], boundary, int(const), None if sum_out is None else C.c_void_p(sum_out.data_ptr()),
           None if max_out is None else C.c_void_p(max_out.data_ptr()), _stream(stream))
    return out


def gray(rgba, out=None, weights=(77, 150, 29), shift=8, stream=None):
    if out is None:
        out = torch.empty(rgba.shape[:-1], dtype=torch.uint8, device=rgba.device)
    vi, vo = view(rgba, rgba=True), view(out)
    L.call("hgb_point_gray", C.byref(vi), C.byref(vo), weights[0], weights[1], weights[2], shift, _stream(stream))
    return out


def binary(op, a, b, out=None, alpha=1.0, beta=1.0, stream=None):
    if out is None:
        out = torch.empty_like(a)
    va, vb, vo = view(a), view(b), view(out)
    L.call("hgb_point_binary", op, C.byref(va), C.byref(vb), C.byref(vo), float(alpha), float(beta),
           _stream(stream))
    return out


def convert(inp, dtype, stream=None):
    out = torch.empty(inp.shape, dtype=dtype, device=inp.device)
    vi, vo = view(inp), view(out)
    L.call("hgb_convert", C.byref(vi), C.byref(vo), _stream(stream))
    return out


INTERPOLATE = {"nn": 1, "lf": 2, "b5": 3, "cf": 4, "l3": 5}  # hipacc::Interpolate numbering


def resample(inp, out, mode="lf", stream=None):
    vi, vo = view(inp), view(out)
    L.call("hgb_resample", C.byref(vi), C.byref(vo), INTERPOLATE[mode], _stream(stream))
    return out


def reduce(inp, op=SUM, win=None, result_dev=None, stream=None):
    """Global reduction; returns the host value (int for integer data, float for floats)."""
    vi = view(inp)
    host = C.create_string_buffer(8)
    L.call("hgb_reduce", C.byref(vi), window(win), op,
           None if result_dev is None else C.c_void_p(result_dev.data_ptr()), host, _stream(stream))
    raw = host.raw
    if inp.dtype in (torch.float32, torch.float16, torch.bfloat16, torch.float64):
        return struct.unpack("<d", raw)[0]
    if inp.dtype in (torch.int16, torch.int32) and op != SUM:
        return struct.unpack("<q", raw)[0]
    if inp.dtype in (torch.int16, torch.int32):
        return struct.unpack("<q", raw)[0]
    return struct.unpack("<Q", raw)[0]


def histogram(inp, num_bins, win=None, bins=None, stream=None):
    """Binned data of the histogram binning function (uint32 bins on the device)."""
    if bins is None:
        bins = torch.empty(num_bins, dtype=torch.int32, device=inp.device)
    vi = view(inp)
    L.call("hgb_histogram", C.byref(vi), window(win), int(num_bins), C.c_void_p(bins.data_ptr()), None,
           _stream(stream))
    return bins


def separable(inp, out=None, row_taps=None, col_taps=None, boundary=CLAMP, const=0.0, stream=None):
    if out is None:
        out = torch.empty_like(inp)
    r = np.ascontiguousarray(row_taps, np.float32)
    c = np.ascontiguousarray(col_taps if col_taps is not None else row_taps, np.float32)
    vi, vo = view(inp), view(out)
    L.call("hgb_separable", C.byref(vi), C.byref(vo), r.ctypes.data_as(C.c_void_p), c.ctypes.data_as(C.c_void_p),
           len(r), boundary, float(const), _stream(stream))
    return out


def bilateral(inp, out=None, smask=None, sigma_r=0.1, boundary=CLAMP, const=0.0, fast_weights=False, stream=None):
    if out is None:
        out = torch.empty_like(inp)
    s = np.ascontiguousarray(smask, np.float32)
    vi, vo = view(inp), view(out)
    L.call("hgb_bilateral", C.byref(vi), C.byref(vo), s.ctypes.data_as(C.c_void_p), s.shape[0], float(sigma_r),
           boundary, float(const), 1 if fast_weights else 0, _stream(stream))
    return out


def set_timing(on: bool) -> None:
    L.call("hgb_set_timing", 1 if on else 0)


def last_kernel_timing() -> float:
    return float(L.load().hgb_last_kernel_timing())


def autotune(on: bool) -> None:
    L.call("hgb_autotune_enable", 1 if on else 0)


class PyramidPlan:
    """Laplacian pyramids of many FP32 images of uneven sizes (hgb_pyramid_plan)."""

    def __init__(self, widths, heights, levels, mask5, boundary=MIRROR):
        import numpy as _np

        self.n = len(widths)
        self.levels = levels
        w = (C.c_int * self.n)(*[int(v) for v in widths])
        h = (C.c_int * self.n)(*[int(v) for v in heights])
        m = _np.ascontiguousarray(mask5, _np.float32)
        self._h = C.c_void_p()
        L.call("hgb_pyramid_plan_create", self.n, w, h, levels, m.ctypes.data_as(C.c_void_p), boundary,
               C.byref(self._h))

    def views(self, image, level):
        g, lap = L.View(), L.View()
        L.call("hgb_pyramid_level_view", self._h, image, level, C.byref(g), C.byref(lap))
        return g, lap

    def _tensor(self, v):
        # a torch view of device memory owned by the plan (rows padded)
        import torch

        if not v.data:
            return None
        n = v.pitch // 4 * v.height
        cuda_arr = _DevicePtr(v.data, n * 4)
        t = torch.as_tensor(cuda_arr, device="cuda").view(torch.float32)
        return t.view(v.height, v.pitch // 4)[:, :v.width]

    def gauss(self, image, level):
        return self._tensor(self.views(image, level)[0])

    def lap(self, image, level):
        return self._tensor(self.views(image, level)[1])

    def decompose(self, mode=0, stream=None):
        L.call("hgb_pyramid_decompose", self._h, mode, _stream(stream))

    def wait_test(self, max_polls=0, kind=0, level=0):
        """Bounded-wait test mode of the plan's launches (hgb_pyramid_plan_wait_test)."""
        L.call("hgb_pyramid_plan_wait_test", self._h, int(max_polls), int(kind), int(level))

    def trace(self, buf=None):
        """Per-CTA records of later single-launch decompositions into `buf` (an
        int64 CUDA tensor of 8 * CTAs), or off with None (hgb_pyramid_plan_trace)."""
        if buf is None:
            L.call("hgb_pyramid_plan_trace", self._h, None, 0)
        else:
            L.call("hgb_pyramid_plan_trace", self._h, C.c_void_p(buf.data_ptr()), buf.numel() // 8)

    def collapse(self, stream=None):
        L.call("hgb_pyramid_collapse", self._h, _stream(stream))

    def close(self):
        if self._h:
            L.call("hgb_pyramid_plan_destroy", self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DevicePtr:
    """__cuda_array_interface__ exporter for plan-owned device memory (bytes)."""

    def __init__(self, ptr, nbytes):
        self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def conv_bilateral_mse(x, t, mask, sigma, smask, boundary=CLAMP, mode=0, stream=None):
    """Forward + adjoint of y1 = conv7x7(x, mask), y = bilateral9x9(y1; smask,
    sigma), loss = mean((y - t)^2).  x, t: (B, H, W) float32 CUDA tensors;
    mask: 7x7 float32 CUDA tensor; sigma: 1-element float32 CUDA tensor.
    Returns (loss [float64, 1], grad_x, grad_mask [7x7], grad_sigma [1])."""
    dev = x.device
    loss = torch.zeros(1, dtype=torch.float64, device=dev)
    gx = torch.empty_like(x)
    gm = torch.empty((7, 7), dtype=torch.float32, device=dev)
    gs = torch.empty(1, dtype=torch.float32, device=dev)
    sm = np.ascontiguousarray(smask, np.float32)
    mask = mask.contiguous()
    vx, vt, vg = view(x), view(t), view(gx)
    L.call("hgb_conv_bilateral_mse", C.byref(vx), C.byref(vt), C.c_void_p(mask.data_ptr()), 7,
           sm.ctypes.data_as(C.c_void_p), 9, C.c_void_p(sigma.data_ptr()), boundary, mode,
           C.c_void_p(loss.data_ptr()), C.byref(vg), C.c_void_p(gm.data_ptr()), C.c_void_p(gs.data_ptr()),
           _stream(stream))
    return loss, gx, gm, gs


def local_op_adjoint(grad_out, mask, boundary=CLAMP, inp=None, want_grad_in=True, want_grad_mask=True, stream=None):
    """Adjoint of the SUM local operator: (grad_in, grad_mask) for a host mask
    (2-D array) or a device mask (2-D float32 CUDA tensor)."""
    gi = torch.empty_like(grad_out) if want_grad_in else None
    if torch.is_tensor(mask):
        mh, mw = mask.shape
        m_host, m_dev = None, C.c_void_p(mask.contiguous().data_ptr())
    else:
        m = np.ascontiguousarray(mask, np.float32)
        mh, mw = m.shape
        m_host, m_dev = m.ctypes.data_as(C.c_void_p), None
    gm = torch.empty((mh, mw), dtype=torch.float32, device=grad_out.device) if want_grad_mask else None
    vg = view(grad_out)
    vi = view(inp) if inp is not None else None
    vgi = view(gi) if gi is not None else None
    L.call("hgb_local_op_adjoint", None if vi is None else C.byref(vi), C.byref(vg),
           None if vgi is None else C.byref(vgi), m_host, m_dev, mw, mh, boundary,
           None if gm is None else C.c_void_p(gm.data_ptr()), _stream(stream))
    return gi, gm


def bilateral_adjoint(inp, grad_out, smask, sigma_r, boundary=CLAMP, const=0.0, want_grad_in=True,
                      want_grad_sigma=True, stream=None):
    """Adjoint of the bilateral filter: (grad_in, grad_sigma [1 float]) for grad_out = dL/dy."""
    gi = torch.empty_like(grad_out) if want_grad_in else None
    gs = torch.zeros(1, dtype=torch.float32, device=inp.device) if want_grad_sigma else None
    s = np.ascontiguousarray(smask, np.float32)
    vi, vg = view(inp), view(grad_out)
    vgi = view(gi) if gi is not None else None
    L.call("hgb_bilateral_adjoint", C.byref(vi), C.byref(vg), s.ctypes.data_as(C.c_void_p), s.shape[0],
           float(sigma_r), boundary, float(const), None if vgi is None else C.byref(vgi),
           None if gs is None else C.c_void_p(gs.data_ptr()), _stream(stream))
    return gi, gs


def separable_adjoint(inp, grad_out, row_taps, col_taps=None, boundary=CLAMP, const=0.0, want_grad_in=True,
                      want_grad_taps=True, stream=None):
    """Adjoint of the separable filter (FP32): (grad_in, grad_row, grad_col)."""
    r = np.ascontiguousarray(row_taps, np.float32)
    c = np.ascontiguousarray(col_taps if col_taps is not None else row_taps, np.float32)
    gi = torch.empty_like(grad_out) if want_grad_in else None
    gr = torch.zeros(len(r), dtype=torch.float32, device=grad_out.device) if want_grad_taps else None
    gc = torch.zeros(len(r), dtype=torch.float32, device=grad_out.device) if want_grad_taps else None
    vi, vg = view(inp), view(grad_out)
    vgi = view(gi) if gi is not None else None
    L.call("hgb_separable_adjoint", C.byref(vi), C.byref(vg), r.ctypes.data_as(C.c_void_p),
           c.ctypes.data_as(C.c_void_p), len(r), boundary, float(const), None if vgi is None else C.byref(vgi),
           None if gr is None else C.c_void_p(gr.data_ptr()), None if gc is None else C.c_void_p(gc.data_ptr()),
           _stream(stream))
    return gi, gr, gc


def minmax_adjoint(inp, grad_out, reduce, mask=None, domain=None, size=None, boundary=CLAMP, const=0.0, stream=None):
    """Adjoint of the MIN / MAX local operator (Domain reduce or convolve with a
    mask): grad_in for grad_out = dL/dout."""
    if mask is not None:
        m = np.ascontiguousarray(mask, np.float32)
        mh, mw = m.shape
        mp = m.ctypes.data_as(C.c_void_p)
    else:
        m, mp = None, None
    if domain is not None:
        d = np.ascontiguousarray(domain, np.uint8)
        mh, mw = d.shape
        dp = d.ctypes.data_as(C.c_void_p)
    else:
        d, dp = None, None
    if m is None and d is None:
        mh = mw = int(size)
    gi = torch.empty_like(grad_out)
    vi, vg, vgi = view(inp), view(grad_out), view(gi)
    L.call("hgb_local_op_minmax_adjoint", C.byref(vi), C.byref(vg), C.byref(vgi), mp, dp, mw, mh, reduce, boundary,
           float(const), _stream(stream))
    return gi


def harris(inp, out=None, k=0.04, threshold=20000.0, boundary=CLAMP, mode=0, stream=None):
    """The Harris corner program (u8 in, 0 / 1 u8 out); mode 0 fused, 1 nine launches."""
    if out is None:
        out = torch.empty_like(inp)
    vi, vo = view(inp), view(out)
    L.call("hgb_harris_corner", C.byref(vi), C.byref(vo), float(k), float(threshold), boundary, mode, _stream(stream))
    return out


def unsharp(rgba, out=None, boundary=CLAMP, mode=0, stream=None):
    """The Unsharp program (uchar4 in and out); mode 0 fused, 1 five launches."""
    if out is None:
        out = torch.empty_like(rgba)
    vi, vo = view(rgba, rgba=True), view(out, rgba=True)
    L.call("hgb_unsharp", C.byref(vi), C.byref(vo), boundary, mode, _stream(stream))
    return out
