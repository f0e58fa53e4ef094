"""TEST INFRASTRUCTURE ONLY: numpy front end of the CPU oracle.

Loads ``oracle/libhgb_oracle.so`` (the C++/OpenMP restatement of Hipacc's CPU
back end, see hgb_oracle.h) and, where it was built in this tree,
``oracle/_ref/libhgb_ref.so`` (the reference's own DSL headers compiled as-is).
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline use this
module; the product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhgb_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libhgb_ref.so")

# hipacc::Boundary (dsl/image.hpp:46-52) and hipacc::Reduce (dsl/kernel.hpp:48-54)
UNDEFINED, CLAMP, REPEAT, MIRROR, CONSTANT = range(5)
SUM, MIN, MAX, PROD = range(4)

_lib = None
_ref = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")


def reference_tree() -> str:
    """Location of the Hipacc source tree as the oracle's Makefile resolves it
    (HIPACC_REF when set); "" when make is unavailable."""
    try:
        r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True, check=True)
    except (OSError, subprocess.CalledProcessError):
        return ""
    return r.stdout.strip()


def build(force: bool = False) -> None:
    """Compile the restated oracle (and the reference pin when the reference tree exists)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle"], check=True)
    tree = reference_tree()
    if tree and os.path.isdir(os.path.join(tree, "dsl")) and (force or not os.path.exists(REF_PATH)):
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_remap.argtypes = [C.c_int] * 4
        L.orc_remap.restype = C.c_int
        L.orc_local_op_f32.argtypes = [f32p, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, f32p, C.c_long,
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int]
        L.orc_local_op_f64.argtypes = [f64p, C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, f64p, C.c_long,
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int]
        L.orc_separable_f32.argtypes = [f32p, C.c_int, C.c_int, f32p, f32p, f32p, C.c_int, C.c_int, C.c_float,
                                        C.c_int, C.c_int]
        L.orc_separable_f64.argtypes = [f64p, C.c_int, C.c_int, f64p, f64p, f64p, C.c_int, C.c_int, C.c_double,
                                        C.c_int]
        L.orc_sobel_mag_u8.argtypes = [u8p, C.c_int, C.c_int, C.c_long, u8p, C.c_long, i32p, i32p, C.c_int,
                                       C.c_int, C.c_int, C.c_int]
        L.orc_rgba_to_gray_u8.argtypes = [u8p, C.c_int, C.c_int, C.c_long, u8p, C.c_long, C.c_int, C.c_int,
                                          C.c_int, C.c_int, C.c_int]
        L.orc_reduce_sum_u8_u64.argtypes = [u8p, C.c_int, C.c_int, C.c_long, C.c_int]
        L.orc_reduce_sum_u8_u64.restype = C.c_uint64
        L.orc_reduce_max_u8.argtypes = [u8p, C.c_int, C.c_int, C.c_long, C.c_int]
        L.orc_reduce_max_u8.restype = C.c_uint32
        L.orc_histogram_f32.argtypes = [f32p, C.c_int, C.c_int, C.c_long, C.c_uint, u32p]
        L.orc_histogram_u8.argtypes = [u8p, C.c_int, C.c_int, C.c_long, C.c_uint, u32p]
        L.orc_reduce_f32.argtypes = [f32p, C.c_int, C.c_int, C.c_long, C.c_int, C.c_int]
        L.orc_reduce_f32.restype = C.c_float
        L.orc_reduce_f32_exact.argtypes = [f32p, C.c_int, C.c_int, C.c_long, C.c_int]
        L.orc_reduce_f32_exact.restype = C.c_double
        L.orc_bilateral_f32.argtypes = [f32p, C.c_int, C.c_int, C.c_long, f32p, C.c_long, f32p, C.c_int,
                                        C.c_float, C.c_int, C.c_float, C.c_int, C.c_int]
        L.orc_bilateral_f64.argtypes = [f64p, C.c_int, C.c_int, C.c_long, f64p, C.c_long, f64p, C.c_int,
                                        C.c_double, C.c_int, C.c_double, C.c_int]
        L.orc_resample_nn_f32.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, C.c_int]
        L.orc_resample_lf_f32.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, C.c_int]
        L.orc_resample_filtered_f32.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_pyramid_decompose_f32.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                                C.c_int, f32p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_pyramid_decompose_f64.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                                C.c_int, f64p, C.c_int, C.c_int, C.c_int]
        L.orc_pyramid_collapse_f32.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                               C.c_int, C.c_int]
        L.orc_c5_loss_f64.argtypes = [f64p, f64p, C.c_int, C.c_int, f64p, C.c_int, f64p, C.c_int, C.c_double,
                                      C.c_int, C.c_int]
        L.orc_c5_loss_f64.restype = C.c_double
        L.orc_c5_grad_f64.argtypes = [f64p, f64p, C.c_int, C.c_int, f64p, C.c_int, f64p, C.c_int, C.c_double,
                                      C.c_int, f64p, f64p, f64p, C.c_int]
        L.orc_c5_grad_f64.restype = C.c_double
        L.orc_bilateral_adjoint_f64.argtypes = [f64p, f64p, C.c_int, C.c_int, f64p, C.c_int, C.c_double, C.c_int,
                                                C.c_double, f64p]
        L.orc_bilateral_adjoint_f64.restype = C.c_double
        L.orc_harris_u8.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, u8p, C.c_int]
        L.orc_unsharp_u8x4.argtypes = [u8p, C.c_int, C.c_int, C.c_int, u8p, C.c_void_p, C.c_int]
        _lib = L
    return _lib


def ref():
    """The reference-built pin library, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = C.CDLL(REF_PATH)
        R.ref_conv_f32.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   f32p]
        R.ref_conv_u8.argtypes = [u8p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, u8p]
        R.ref_sobel_mag_u8.argtypes = [u8p, C.c_int, C.c_int, i32p, i32p, C.c_int, C.c_int, u8p]
        R.ref_gray_u8.argtypes = [u8p, C.c_int, C.c_int, u8p]
        R.ref_sum_u8_u64.argtypes = [u8p, C.c_int, C.c_int]
        R.ref_sum_u8_u64.restype = C.c_uint64
        R.ref_max_u8.argtypes = [u8p, C.c_int, C.c_int]
        R.ref_max_u8.restype = C.c_uint32
        R.ref_reduce_f32.argtypes = [f32p, C.c_int, C.c_int, C.c_int]
        R.ref_reduce_f32.restype = C.c_float
        R.ref_bilateral_f32.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_float, C.c_int, f32p]
        R.ref_resample_f32.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, C.c_int]
        R.ref_pyramid_f32.argtypes = [f32p, C.c_int, C.c_int, C.c_int, f32p, C.c_int, f32p, f32p]
        for n in ("ref_cpu_red_sum_f32_serial", "ref_cpu_red_max_f32_serial", "ref_cpu_red_sum_f32_omp",
                  "ref_cpu_red_max_f32_omp"):
            getattr(R, n).argtypes = [f32p, C.c_int, C.c_int]
            getattr(R, n).restype = C.c_float
        R.ref_cpu_red_cores_omp.restype = C.c_int
        R.ref_harris_u8.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, u8p]
        R.ref_unsharp_u8x4.argtypes = [u8p, C.c_int, C.c_int, C.c_int, u8p, C.c_void_p]
        R.ref_cpu_interp_f32.argtypes = [C.c_int, f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int]
        for n in ("ref_cpu_histogram_f32_serial", "ref_cpu_histogram_f32_omp"):
            getattr(R, n).argtypes = [f32p, C.c_int, C.c_int, C.c_uint, u32p]
        _ref = R
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def remap(mode, idx, lo, hi):
    return lib().orc_remap(mode, idx, lo, hi)


def local_op(img, mask=None, domain=None, size=None, reduce=SUM, boundary=CLAMP, const=0.0, contract=1,
             acc=None, out=None, iter_space=None, nthreads=0):
    """Generic local operator.  ``img`` float32/float64 (h, w).  ``acc`` is the
    Accessor window (ox, oy, w, h) on img; ``iter_space`` the IterationSpace
    window on ``out`` (default: a fresh array of the accessor's size)."""
    img = np.ascontiguousarray(img)
    dt = img.dtype
    assert dt in (np.float32, np.float64)
    h, w = img.shape
    if mask is not None:
        mask = np.ascontiguousarray(mask, dtype=dt)
        mh, mw = mask.shape
    else:
        mh, mw = size if size is not None else np.asarray(domain).shape
    if domain is not None:
        domain = np.ascontiguousarray(domain, dtype=np.uint8)
    aox, aoy, aw, ah = acc if acc is not None else (0, 0, w, h)
    if out is None:
        out = np.zeros((ah, aw), dtype=dt)
    ioh, iow = out.shape
    iox, ioy, iw, ih = iter_space if iter_space is not None else (0, 0, aw, ah)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    fn = lib().orc_local_op_f32 if dt == np.float32 else lib().orc_local_op_f64
    fn(img, w, aox, aoy, aw, ah, out, iow, iox, ioy, iw, ih, _ptr(mask), _ptr(domain), mw, mh, reduce,
       boundary, const, contract, nt)
    return out


def write_u8(v):
    """A float result written to a u8 image as the image samples write it,
    ``(uchar)(v + 0.5f)`` (samples-public/1_Local_Operators/Gaussian_Blur/src/main.cpp),
    in FP32; values outside [0, 255] saturate where C leaves the cast undefined
    (NaN gives 255: the kernels clamp with fminf, which returns the number)."""
    s = (np.asarray(v, np.float32) + np.float32(0.5)).astype(np.float32)
    s = np.nan_to_num(s, nan=255.0, posinf=255.0, neginf=0.0)
    return np.clip(np.trunc(s), 0, 255).astype(np.uint8)


def local_op_u8(img, mask=None, domain=None, size=None, reduce=SUM, boundary=CLAMP, const=0.0, contract=1, **kw):
    """A local operator on a u8 image: the FP32 operator on the widened pixels,
    written back with ``write_u8``."""
    r = local_op(np.asarray(img).astype(np.float32), mask=mask, domain=domain, size=size, reduce=reduce,
                 boundary=boundary, const=const, contract=contract, **kw)
    return write_u8(r)


def separable(img, row_taps, col_taps, boundary=CLAMP, const=0.0, contract=1, nthreads=0):
    img = np.ascontiguousarray(img)
    h, w = img.shape
    out = np.zeros_like(img)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    k = len(row_taps)
    if img.dtype == np.float32:
        lib().orc_separable_f32(img, w, h, out, np.ascontiguousarray(row_taps, np.float32),
                                np.ascontiguousarray(col_taps, np.float32), k, boundary, const, contract, nt)
    else:
        lib().orc_separable_f64(img, w, h, out, np.ascontiguousarray(row_taps, np.float64),
                                np.ascontiguousarray(col_taps, np.float64), k, boundary, const, nt)
    return out


SOBEL3_X = np.array([[-1, 0, 1], [-2, 0, 2], [-1, 0, 1]], np.int32)
SOBEL3_Y = np.array([[-1, -2, -1], [0, 0, 0], [1, 2, 1]], np.int32)


def sobel_mag(img, mask_x=SOBEL3_X, mask_y=SOBEL3_Y, boundary=MIRROR, const=0, nthreads=0):
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape
    out = np.zeros_like(img)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    lib().orc_sobel_mag_u8(img, w, h, w, out, w, np.ascontiguousarray(mask_x, np.int32),
                           np.ascontiguousarray(mask_y, np.int32), mask_x.shape[0], boundary, const, nt)
    return out


def rgba_to_gray(rgba, weights=(77, 150, 29), shift=8, nthreads=0):
    rgba = np.ascontiguousarray(rgba, np.uint8)
    h, w = rgba.shape[:2]
    out = np.zeros((h, w), np.uint8)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    lib().orc_rgba_to_gray_u8(rgba.reshape(h, w * 4), w, h, w, out, w, weights[0], weights[1], weights[2], shift,
                              nt)
    return out


def reduce_sum_u8(img, nthreads=1):
    img = np.ascontiguousarray(img, np.uint8)
    return int(lib().orc_reduce_sum_u8_u64(img, img.shape[1], img.shape[0], img.shape[1], nthreads))


def reduce_max_u8(img, nthreads=1):
    img = np.ascontiguousarray(img, np.uint8)
    return int(lib().orc_reduce_max_u8(img, img.shape[1], img.shape[0], img.shape[1], nthreads))


def histogram(img, num_bins):
    """Binned data of the histogram sample's binning function (u32 bins)."""
    bins = np.zeros(num_bins, np.uint32)
    if img.dtype == np.uint8:
        img = np.ascontiguousarray(img)
        lib().orc_histogram_u8(img, img.shape[1], img.shape[0], img.shape[1], num_bins, bins)
    else:
        img = np.ascontiguousarray(img, np.float32)
        lib().orc_histogram_f32(img, img.shape[1], img.shape[0], img.shape[1], num_bins, bins)
    return bins


def reduce_f32(img, op=SUM, nthreads=1):
    img = np.ascontiguousarray(img, np.float32)
    return float(lib().orc_reduce_f32(img, img.shape[1], img.shape[0], img.shape[1], op, nthreads))


def reduce_f32_exact(img, op=SUM):
    img = np.ascontiguousarray(img, np.float32)
    return float(lib().orc_reduce_f32_exact(img, img.shape[1], img.shape[0], img.shape[1], op))


def bilateral(img, smask, sigma_r, boundary=CLAMP, const=0.0, contract=1, nthreads=0):
    img = np.ascontiguousarray(img)
    h, w = img.shape
    out = np.zeros_like(img)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    size = smask.shape[0]
    if img.dtype == np.float32:
        lib().orc_bilateral_f32(img, w, h, w, out, w, np.ascontiguousarray(smask, np.float32), size, sigma_r,
                                boundary, const, contract, nt)
    else:
        lib().orc_bilateral_f64(img, w, h, w, out, w, np.ascontiguousarray(smask, np.float64), size, sigma_r,
                                boundary, const, nt)
    return out


FILTERED = {"b5": 3, "cf": 4, "l3": 5}


def resample_filtered(src, dw, dh, mode, contract=1):
    """B5 / CF / L3 resampling accessors of the CPU back end (clamped taps)."""
    src = np.ascontiguousarray(src, np.float32)
    dst = np.zeros((dh, dw), np.float32)
    lib().orc_resample_filtered_f32(src, src.shape[1], src.shape[0], dst, dw, dh, FILTERED[mode], contract)
    return dst


def resample(src, dw, dh, mode="lf", contract=1):
    src = np.ascontiguousarray(src, np.float32)
    sh, sw = src.shape
    dst = np.zeros((dh, dw), np.float32)
    fn = lib().orc_resample_lf_f32 if mode == "lf" else lib().orc_resample_nn_f32
    fn(src, sw, sh, dst, dw, dh, contract)
    return dst


def level_sizes(w, h, levels):
    sizes = [(w, h)]
    for _ in range(1, levels):
        w, h = w // 2, h // 2
        sizes.append((w, h))
    return sizes


def pyramid_decompose(img, levels, mask, boundary=MIRROR, contract=1, nthreads=0):
    """Returns (gauss levels, laplacian levels) as lists of arrays."""
    img = np.ascontiguousarray(img)
    dt = img.dtype
    h, w = img.shape
    sizes = level_sizes(w, h, levels)
    gauss = [img.copy()] + [np.zeros((sh, sw), dt) for (sw, sh) in sizes[1:]]
    lap = [np.zeros((sh, sw), dt) for (sw, sh) in sizes[:-1]]
    gp = (C.c_void_p * levels)(*[g.ctypes.data for g in gauss])
    lp = (C.c_void_p * max(1, levels - 1))(*[a.ctypes.data for a in lap])
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    m = np.ascontiguousarray(mask, dt)
    if dt == np.float32:
        lib().orc_pyramid_decompose_f32(gp, lp, w, h, levels, m, m.shape[0], boundary, contract, nt)
    else:
        lib().orc_pyramid_decompose_f64(gp, lp, w, h, levels, m, m.shape[0], boundary, nt)
    return gauss, lap


def pyramid_collapse(bottom, lap, contract=1):
    levels = len(lap) + 1
    h, w = lap[0].shape
    sizes = level_sizes(w, h, levels)
    outs = [np.zeros((sh, sw), np.float32) for (sw, sh) in sizes]
    outs[-1][...] = bottom
    op = (C.c_void_p * levels)(*[o.ctypes.data for o in outs])
    lp = (C.c_void_p * max(1, levels - 1))(*[np.ascontiguousarray(a).ctypes.data for a in lap])
    lib().orc_pyramid_collapse_f32(op, lp, w, h, levels, contract)
    return outs


def c5_loss(x, t, mask, smask, sigma_r, boundary=CLAMP, nthreads=0):
    x = np.ascontiguousarray(x, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    h, w = x.shape
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    return float(lib().orc_c5_loss_f64(x, t, w, h, np.ascontiguousarray(mask, np.float64), mask.shape[0],
                                       np.ascontiguousarray(smask, np.float64), smask.shape[0], sigma_r, boundary,
                                       nt))


def c5_grad(x, t, mask, smask, sigma_r, boundary=CLAMP, nthreads=0):
    x = np.ascontiguousarray(x, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    h, w = x.shape
    dx = np.zeros_like(x)
    dmask = np.zeros(mask.shape, np.float64)
    dsig = np.zeros(1, np.float64)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    loss = lib().orc_c5_grad_f64(x, t, w, h, np.ascontiguousarray(mask, np.float64), mask.shape[0],
                                 np.ascontiguousarray(smask, np.float64), smask.shape[0], sigma_r, boundary, dx,
                                 dmask, dsig, nt)
    return float(loss), dx, dmask, float(dsig[0])


def harris(img, boundary=CLAMP, k=0.04, threshold=20000.0, nthreads=0):
    """The Harris corner sample's program (3x3): 0 / 1 per pixel."""
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape
    out = np.zeros((h, w), np.uint8)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    lib().orc_harris_u8(img, w, h, boundary, k, threshold, out, nt)
    return out


def unsharp(rgba, boundary=CLAMP, nthreads=0):
    """The Unsharp sample's program (3x3): (uchar4 output, luminance)."""
    rgba = np.ascontiguousarray(rgba, np.uint8)
    h, w = rgba.shape[:2]
    out = np.zeros((h, w, 4), np.uint8)
    gray = np.zeros((h, w), np.float32)
    nt = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    lib().orc_unsharp_u8x4(rgba.reshape(h, w * 4), w, h, boundary, out.reshape(h, w * 4), gray.ctypes.data_as(C.c_void_p),
                           nt)
    return out, gray


def bilateral_adjoint(img, grad_out, smask, sigma_r, boundary=CLAMP, const=0.0):
    """FP64 adjoint of the bilateral filter: (dL/din, dL/dsigma_r) for dL/dy = grad_out."""
    x = np.ascontiguousarray(img, np.float64)
    g = np.ascontiguousarray(grad_out, np.float64)
    h, w = x.shape
    gi = np.zeros_like(x)
    ds = lib().orc_bilateral_adjoint_f64(x, g, w, h, np.ascontiguousarray(smask, np.float64), smask.shape[0],
                                         float(sigma_r), boundary, float(const), gi)
    return gi, float(ds)


def remap_vec(mode, idx, n):
    """remap() over an index vector; negative where CONSTANT reads the constant."""
    return np.array([remap(mode, int(i), 0, n) for i in idx], np.int64)


def local_op_adjoint(img, grad_out, mask, boundary=CLAMP):
    """FP64 adjoint of the SUM local operator out(j) = sum_o m_o in(r(j + o))
    (lib/AST/Convolution.cpp:43-100 with the remap of
    lib/AST/BorderHandling.cpp:41-120), by scattering: every tap o of every
    output j sends m_o grad_out(j) to r(j + o); CONSTANT taps send nothing and
    read 0 in the mask gradient.  Returns (grad_in, grad_mask)."""
    gout = np.asarray(grad_out, np.float64)
    img = np.asarray(img, np.float64)
    mask = np.asarray(mask)
    h, w = gout.shape
    mh, mw = mask.shape
    gin = np.zeros((h, w))
    gm = np.zeros((mh, mw))
    ys, xs = np.arange(h), np.arange(w)
    for my in range(mh):
        ry = remap_vec(boundary, ys + my - mh // 2, h)
        for mx in range(mw):
            rx = remap_vec(boundary, xs + mx - mw // 2, w)
            Y, X = np.meshgrid(np.where(ry >= 0)[0], np.where(rx >= 0)[0], indexing="ij")
            np.add.at(gin, (ry[Y], rx[X]), float(mask[my, mx]) * gout[Y, X])
            gm[my, mx] = np.sum(gout[Y, X] * img[ry[Y], rx[X]])
    return gin, gm


def separable_adjoint(img, grad_out, row_taps, col_taps, boundary=CLAMP, const=0.0):
    """FP64 adjoint of the separable filter t = rows(in), out = cols(t), each a
    1-D SUM local operator with the boundary (rows of t outside the image are
    t's own remap, or the constant).  Returns (grad_in, grad_row, grad_col);
    the tap gradients count CONSTANT taps outside as reading 0."""
    x = np.asarray(img, np.float64)
    h, w = x.shape
    k = len(row_taps)
    t = np.zeros((h, w))
    xs = np.arange(w)
    for j in range(k):
        rx = remap_vec(boundary, xs + j - k // 2, w)
        t += float(row_taps[j]) * np.where((rx >= 0)[None, :], x[:, np.clip(rx, 0, w - 1)], const)
    gt, gcol = local_op_adjoint(t, grad_out, np.asarray(col_taps).reshape(-1, 1), boundary)
    gin, grow = local_op_adjoint(x, gt, np.asarray(row_taps).reshape(1, -1), boundary)
    return gin, grow.ravel(), gcol.ravel()


def minmax_adjoint(img, grad_out, reduce, mask=None, domain=None, boundary=CLAMP, const=0.0):
    """The MIN / MAX local operator and its adjoint.  Forward as the reference
    evaluates it (lib/AST/Convolution.cpp:43-100, dsl/math_functions.hpp:347-376):
    acc starts at FLT_MAX (MIN) or FLT_MIN (MAX), and every tap of the Domain
    (or of the mask, v = m * x in float32 for convolve) in row-major order takes
    acc = acc < v ? acc : v or acc > v ? acc : v.  The gradient of an output
    goes to the pixel read by the tap that last replaced the running value
    (times its mask weight); nothing when no tap replaced the start value or
    when the winner read the CONSTANT value outside.  Returns (out as float32,
    grad_in in FP64)."""
    img = np.asarray(img, np.float32)
    h, w = img.shape
    shape = np.asarray(mask if mask is not None else domain).shape
    mh, mw = shape
    is_max = reduce == MAX
    acc = np.full((h, w), np.finfo(np.float32).tiny if is_max else np.finfo(np.float32).max, np.float32)
    win = np.full((h, w), -1, np.int64)
    sy = np.zeros((h, w), np.int64)
    sx = np.zeros((h, w), np.int64)
    ys, xs = np.arange(h), np.arange(w)
    for my in range(mh):
        ry = remap_vec(boundary, ys + my - mh // 2, h)
        for mx in range(mw):
            if domain is not None and not domain[my][mx]:
                continue
            rx = remap_vec(boundary, xs + mx - mw // 2, w)
            outside = (ry[:, None] < 0) | (rx[None, :] < 0)
            RY = np.broadcast_to(np.clip(ry, 0, h - 1)[:, None], (h, w))
            RX = np.broadcast_to(np.clip(rx, 0, w - 1)[None, :], (h, w))
            xv = np.where(outside, np.float32(const), img[RY, RX]).astype(np.float32)
            v = (np.float32(mask[my][mx]) * xv).astype(np.float32) if mask is not None else xv
            upd = ~(acc > v) if is_max else ~(acc < v)
            acc = np.where(upd, v, acc)
            win = np.where(upd, np.where(outside, -1, my * mw + mx), win)
            sy = np.where(upd, RY, sy)
            sx = np.where(upd, RX, sx)
    gin = np.zeros((h, w))
    ok = win >= 0
    fac = np.ones(win.shape) if mask is None else np.asarray(mask, np.float64).ravel()[np.maximum(win, 0)]
    np.add.at(gin, (sy[ok], sx[ok]), (fac * np.asarray(grad_out, np.float64))[ok])
    return acc, gin


# ---- standard masks (FP64 construction rounded once to FP32) ----

def gaussian_mask(size, sigma, dtype=np.float32):
    """Normalised 2-D Gaussian exp(-(x^2+y^2)/(2 sigma^2)) built in FP64, rounded once."""
    r = size // 2
    ax = np.arange(-r, r + 1, dtype=np.float64)
    g = np.exp(-(ax[None, :] ** 2 + ax[:, None] ** 2) / (2.0 * sigma * sigma))
    g /= g.sum()
    return g.astype(dtype)


def gaussian_taps(size, sigma, dtype=np.float32):
    r = size // 2
    ax = np.arange(-r, r + 1, dtype=np.float64)
    g = np.exp(-(ax ** 2) / (2.0 * sigma * sigma))
    g /= g.sum()
    return g.astype(dtype)


def spatial_mask(size, sigma_d, dtype=np.float32):
    """Bilateral spatial weights exp(-(x^2+y^2)/(2 sigma_d^2)), centre 1, built in FP64."""
    r = size // 2
    ax = np.arange(-r, r + 1, dtype=np.float64)
    g = np.exp(-(ax[None, :] ** 2 + ax[:, None] ** 2) / (2.0 * sigma_d * sigma_d))
    return g.astype(dtype)


def binomial5(dtype=np.float32):
    a = np.array([1, 4, 6, 4, 1], np.float64) / 16.0
    return np.outer(a, a).astype(dtype)
