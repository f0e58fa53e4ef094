"""Generate tests/golden/*.npz from the reference's own DSL headers.

Run in a tree where the reference sources exist (the oracle Makefile's `ref`
target compiles dsl/*.hpp and runtime/hipacc_cpu_red.hpp of the reference as-is
into oracle/_ref/libhgb_ref.so).  Every fixture holds the seeded inputs and the
outputs the reference computed; tests/test_oracle_golden.py checks the
restated oracle against them wherever the reference tree is absent.

DSL mode ignores the CONSTANT value (dsl/image.hpp:260-291), so CONSTANT
fixtures use the constant 0, where both agree.  Floating-point fixtures are
compiled with -ffp-contract=off (no fused multiply-add).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402


def blocks_u8(rng, h, w, n=12, noise=6):
    """Random axis-aligned rectangles of random grey levels plus uniform noise."""
    img = np.full((h, w), int(rng.integers(0, 256)), np.int32)
    for _ in range(n):
        y0, x0 = int(rng.integers(0, h - 2)), int(rng.integers(0, w - 2))
        y1, x1 = int(rng.integers(y0 + 2, h + 1)), int(rng.integers(x0 + 2, w + 1))
        img[y0:y1, x0:x1] = int(rng.integers(0, 256))
    img += rng.integers(-noise, noise + 1, (h, w))
    return np.clip(img, 0, 255).astype(np.uint8)


def main():
    O.build()
    R = O.ref()
    if R is None:
        raise SystemExit("oracle/_ref/libhgb_ref.so is not built (needs the reference tree)")
    rng = np.random.default_rng(20261203)
    out = {}

    # local operators: Kernel::convolve with a Mask, all boundary modes
    for (mh, mw) in [(3, 3), (5, 5), (1, 9), (9, 1), (13, 13)]:
        for b in (O.CLAMP, O.REPEAT, O.MIRROR, O.CONSTANT):
            h, w = 19, 23
            img = rng.random((h, w), dtype=np.float32)
            m = rng.random((mh, mw)).astype(np.float32)
            r = np.zeros_like(img)
            assert R.ref_conv_f32(img, w, h, m, mw, mh, b, 0, 0, r) == 0
            out[f"conv_{mh}x{mw}_b{b}_in"] = img
            out[f"conv_{mh}x{mw}_b{b}_mask"] = m
            out[f"conv_{mh}x{mw}_b{b}_out"] = r
    # Kernel::reduce over a Domain (SUM / MIN / MAX)
    for red in (O.SUM, O.MIN, O.MAX):
        h, w = 17, 21
        img = rng.random((h, w), dtype=np.float32)
        dom = (rng.random((5, 5)) > 0.35).astype(np.float32)
        r = np.zeros_like(img)
        R.ref_conv_f32(img, w, h, dom, 5, 5, O.MIRROR, 1, red, r)
        out[f"domain_r{red}_in"] = img
        out[f"domain_r{red}_dom"] = dom.astype(np.uint8)
        out[f"domain_r{red}_out"] = r
    # Sobel magnitude over Domains, u8, every boundary mode
    for b in (O.CLAMP, O.REPEAT, O.MIRROR, O.CONSTANT):
        img = rng.integers(0, 256, (21, 37), dtype=np.uint8)
        r = np.zeros_like(img)
        R.ref_sobel_mag_u8(img, 37, 21, O.SOBEL3_X, O.SOBEL3_Y, 3, b, r)
        out[f"sobel_b{b}_in"] = img
        out[f"sobel_b{b}_out"] = r
    # RGBA -> gray
    rgba = rng.integers(0, 256, (13, 29, 4), dtype=np.uint8)
    g = np.zeros((13, 29), np.uint8)
    R.ref_gray_u8(rgba, 29, 13, g)
    out["gray_in"] = rgba
    out["gray_out"] = g
    # reductions
    img = rng.integers(0, 256, (31, 45), dtype=np.uint8)
    out["red_u8_in"] = img
    out["red_u8_sum"] = np.array([R.ref_sum_u8_u64(img, 45, 31)], np.uint64)
    out["red_u8_max"] = np.array([R.ref_max_u8(img, 45, 31)], np.uint32)
    f = rng.random((29, 33), dtype=np.float32)
    out["red_f32_in"] = f
    out["red_f32_dsl"] = np.array([R.ref_reduce_f32(f, 33, 29, op) for op in (0, 1, 2)], np.float32)
    out["red_f32_cpu2d_serial"] = np.array([R.ref_cpu_red_sum_f32_serial(f, 33, 29)], np.float32)
    # bilateral (sample body with float sigma_r)
    for size in (5, 13):
        img = rng.random((18, 22), dtype=np.float32)
        sm = O.spatial_mask(size, 3.0)
        r = np.zeros_like(img)
        R.ref_bilateral_f32(img, 22, 18, sm, size, 0.1, O.CLAMP, r)
        out[f"bilateral_{size}_in"] = img
        out[f"bilateral_{size}_mask"] = sm
        out[f"bilateral_{size}_out"] = r
    # NN / LF accessors
    for (sw, sh, dw, dh) in [(37, 29, 18, 14), (18, 14, 37, 29)]:
        src = rng.random((sh, sw), dtype=np.float32)
        for mode, im in (("nn", 1), ("lf", 2)):
            r = np.zeros((dh, dw), np.float32)
            R.ref_resample_f32(src, sw, sh, r, dw, dh, im)
            out[f"resample_{mode}_{sw}x{sh}_{dw}x{dh}_in"] = src
            out[f"resample_{mode}_{sw}x{sh}_{dw}x{dh}_out"] = r
    # Laplacian pyramid through Pyramid / traverse
    w, h, L = 67, 45, 4
    img = rng.random((h, w), dtype=np.float32)
    sizes = O.level_sizes(w, h, L)
    go = np.zeros(sum(a * b for a, b in sizes), np.float32)
    lo = np.zeros(sum(a * b for a, b in sizes[:-1]), np.float32)
    R.ref_pyramid_f32(img, w, h, L, O.binomial5(), O.MIRROR, go, lo)
    out["pyramid_in"] = img
    out["pyramid_gauss"] = go
    out["pyramid_lap"] = lo
    path = os.path.join(HERE, "hipacc_ref_golden.npz")
    # binning: the histogram sample's binning function through BINNING_CPU_2D
    hist = (rng.random((29, 41)) * 255.0).astype(np.float32)
    hist[0, :3] = [255.0, 0.0, 254.999]
    out["hist_in"] = hist
    for nb in (7, 64, 256, 1000):
        bins = np.zeros(nb, np.uint32)
        R.ref_cpu_histogram_f32_serial(hist, 41, 29, nb, bins)
        out[f"hist_{nb}"] = bins
    # B5 / CF / L3 resampling accessors through the CPU back end's own macros
    for (sh, sw, dh, dw) in ((17, 23, 40, 31), (30, 50, 11, 19)):
        src = rng.random((sh, sw), dtype=np.float32)
        out[f"interp_{sw}x{sh}_{dw}x{dh}_in"] = src
        for name, m in (("b5", 3), ("cf", 4), ("l3", 5)):
            dst = np.zeros((dh, dw), np.float32)
            assert R.ref_cpu_interp_f32(m, src, sw, sh, dst, dw, dh) == 0
            out[f"interp_{name}_{sw}x{sh}_{dw}x{dh}"] = dst
    # u8 images: the Gaussian-blur sample's (uchar)(convolve(...) + 0.5f) and
    # the Erode / Dilate samples' reduce(dom, MIN / MAX) over uchar
    for (mh, mw) in [(3, 3), (5, 5), (1, 5), (5, 1)]:
        for b in (O.CLAMP, O.REPEAT, O.MIRROR, O.CONSTANT):
            img = rng.integers(0, 256, (19, 23), dtype=np.uint8)
            m = rng.random((mh, mw)).astype(np.float32)
            m /= m.sum()
            r = np.zeros_like(img)
            assert R.ref_conv_u8(img, 23, 19, m, mw, mh, b, 0, 0, r) == 0
            out[f"conv_u8_{mh}x{mw}_b{b}_in"] = img
            out[f"conv_u8_{mh}x{mw}_b{b}_mask"] = m
            out[f"conv_u8_{mh}x{mw}_b{b}_out"] = r
    for red in (O.MIN, O.MAX):
        img = rng.integers(0, 256, (17, 21), dtype=np.uint8)
        dom = np.ones((3, 3), np.float32)
        dom[0, 0] = dom[2, 2] = 0.0
        r = np.zeros_like(img)
        assert R.ref_conv_u8(img, 21, 17, dom, 3, 3, O.CLAMP, 1, red, r) == 0
        out[f"domain_u8_r{red}_in"] = img
        out[f"domain_u8_r{red}_dom"] = dom.astype(np.uint8)
        out[f"domain_u8_r{red}_out"] = r
    # the Harris corner and Unsharp sample programs (3x3) on structured images:
    # random rectangles plus noise give corners, edges and flat regions
    for b in (O.CLAMP, O.REPEAT, O.MIRROR):
        img = blocks_u8(rng, 40, 56)
        r = np.zeros_like(img)
        R.ref_harris_u8(img, 56, 40, b, 0.04, 20000.0, r)
        out[f"harris_b{b}_in"] = img
        out[f"harris_b{b}_out"] = r
        rgba = np.stack([blocks_u8(rng, 33, 47) for _ in range(4)], axis=-1)
        ro = np.zeros_like(rgba)
        rg = np.zeros((33, 47), np.float32)
        R.ref_unsharp_u8x4(rgba.reshape(33, 47 * 4), 47, 33, b, ro.reshape(33, 47 * 4), rg.ctypes.data_as(C.c_void_p))
        out[f"unsharp_b{b}_in"] = rgba
        out[f"unsharp_b{b}_out"] = ro
        out[f"unsharp_b{b}_gray"] = rg
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
