"""CPU: the restated oracle against the reference's own DSL results.

tests/golden/hipacc_ref_golden.npz was produced by tests/golden/make_golden.py
from the reference's dsl/*.hpp and runtime/hipacc_cpu_red.hpp compiled as-is.
Where the reference tree is present, the same checks also run live against
oracle/_ref on fresh random inputs.
"""
import numpy as np
import pytest


def test_conv_golden(oracle, golden):
    O = oracle
    n = 0
    for (mh, mw) in [(3, 3), (5, 5), (1, 9), (9, 1), (13, 13)]:
        for b in (O.CLAMP, O.REPEAT, O.MIRROR, O.CONSTANT):
            k = f"conv_{mh}x{mw}_b{b}"
            r = O.local_op(golden[k + "_in"], mask=golden[k + "_mask"], boundary=b, const=0.0, contract=0)
            assert np.array_equal(r, golden[k + "_out"]), k
            n += 1
    assert n == 20


def test_domain_golden(oracle, golden):
    O = oracle
    for red in (O.SUM, O.MIN, O.MAX):
        k = f"domain_r{red}"
        dom = golden[k + "_dom"]
        r = O.local_op(golden[k + "_in"], domain=dom, size=dom.shape, reduce=red, boundary=O.MIRROR, contract=0)
        assert np.array_equal(r, golden[k + "_out"]), k


def test_u8_local_op_golden(oracle, golden):
    """u8 images through the reference's DSL: the Gaussian-blur sample's
    (uchar)(convolve + 0.5f) and the Erode / Dilate samples' reduce(dom, MIN / MAX)."""
    O = oracle
    n = 0
    for (mh, mw) in [(3, 3), (5, 5), (1, 5), (5, 1)]:
        for b in (O.CLAMP, O.REPEAT, O.MIRROR, O.CONSTANT):
            k = f"conv_u8_{mh}x{mw}_b{b}"
            r = O.local_op_u8(golden[k + "_in"], mask=golden[k + "_mask"], boundary=b, const=0.0, contract=0)
            assert np.array_equal(r, golden[k + "_out"]), k
            n += 1
    for red in (O.MIN, O.MAX):
        k = f"domain_u8_r{red}"
        dom = golden[k + "_dom"]
        r = O.local_op_u8(golden[k + "_in"], domain=dom, size=dom.shape, reduce=red, boundary=O.CLAMP, contract=0)
        assert np.array_equal(r, golden[k + "_out"]), k
        n += 1
    assert n == 18


def test_write_u8_rule(oracle):
    """(uchar)(v + 0.5f) for in-range values; saturation outside.  The sum is
    rounded in FP32 first: 0.49999997f + 0.5f lies halfway between 1 - 2^-24
    and 1 and rounds to 1, as the sample's C expression does."""
    v = np.array([0.0, 0.49999997, 0.5, 1.49, 254.5, 254.49998, 255.2, 300.0, -0.4, -3.0], np.float32)
    assert oracle.write_u8(v).tolist() == [0, 1, 1, 1, 255, 254, 255, 255, 0, 0]


def test_sobel_gray_reduce_golden(oracle, golden):
    O = oracle
    for b in (O.CLAMP, O.REPEAT, O.MIRROR, O.CONSTANT):
        assert np.array_equal(O.sobel_mag(golden[f"sobel_b{b}_in"], boundary=b), golden[f"sobel_b{b}_out"])
    assert np.array_equal(O.rgba_to_gray(golden["gray_in"]), golden["gray_out"])
    img = golden["red_u8_in"]
    assert O.reduce_sum_u8(img) == int(golden["red_u8_sum"][0])
    assert O.reduce_max_u8(img) == int(golden["red_u8_max"][0])
    f = golden["red_f32_in"]
    for i, op in enumerate((O.SUM, O.MIN, O.MAX)):
        assert np.float32(O.reduce_f32(f, op, 1)) == golden["red_f32_dsl"][i]
    assert np.float32(O.reduce_f32(f, O.SUM, 1)) == golden["red_f32_cpu2d_serial"][0]


def test_histogram_golden(oracle, golden):
    """Binning: the restated histogram against the reference's BINNING_CPU_2D
    with the histogram sample's binning function (255.0 lands past the last
    bin and is dropped)."""
    img = golden["hist_in"]
    for nb in (7, 64, 256, 1000):
        assert np.array_equal(oracle.histogram(img, nb), golden[f"hist_{nb}"])
    u8 = img.astype(np.uint8)
    assert np.array_equal(oracle.histogram(u8, 256), oracle.histogram(u8.astype(np.float32), 256))


def test_filtered_resampling_golden(oracle, golden):
    """B5 / CF / L3 accessors: the restatement against the CPU back end's own
    macros (including the Lanczos weight the reference gives the fifth tap of
    the second row)."""
    for (sh, sw, dh, dw) in ((17, 23, 40, 31), (30, 50, 11, 19)):
        src = golden[f"interp_{sw}x{sh}_{dw}x{dh}_in"]
        for mode in ("b5", "cf", "l3"):
            got = oracle.resample_filtered(src, dw, dh, mode, contract=0)
            assert np.array_equal(got, golden[f"interp_{mode}_{sw}x{sh}_{dw}x{dh}"]), mode


def test_bilateral_golden(oracle, golden):
    O = oracle
    for size in (5, 13):
        k = f"bilateral_{size}"
        r = O.bilateral(golden[k + "_in"], golden[k + "_mask"], 0.1, boundary=O.CLAMP, contract=0)
        assert np.array_equal(r, golden[k + "_out"]), k


def test_resample_pyramid_golden(oracle, golden):
    O = oracle
    for (sw, sh, dw, dh) in [(37, 29, 18, 14), (18, 14, 37, 29)]:
        for mode in ("nn", "lf"):
            k = f"resample_{mode}_{sw}x{sh}_{dw}x{dh}"
            assert np.array_equal(O.resample(golden[k + "_in"], dw, dh, mode, contract=0), golden[k + "_out"]), k
    g, lap = O.pyramid_decompose(golden["pyramid_in"], 4, O.binomial5(), O.MIRROR, contract=0)
    assert np.array_equal(np.concatenate([a.ravel() for a in g]), golden["pyramid_gauss"])
    assert np.array_equal(np.concatenate([a.ravel() for a in lap]), golden["pyramid_lap"])


def test_contraction_is_within_reference_tolerance(oracle):
    """The FMA-contracted form (what nvcc and aarch64 GCC emit) stays within
    1e-6 relative of the separately rounded form on a 5x5 Gaussian."""
    O = oracle
    rng = np.random.default_rng(5)
    img = rng.random((64, 80), dtype=np.float32)
    m = O.gaussian_mask(5, 1.0)
    a = O.local_op(img, mask=m, boundary=O.CLAMP, contract=1)
    b = O.local_op(img, mask=m, boundary=O.CLAMP, contract=0)
    assert np.max(np.abs(a - b) / np.abs(b)) <= 1e-6


def test_remap_rules(oracle):
    O = oracle
    # lib/AST/BorderHandling.cpp:41-120 on a window [2, 7)
    assert [O.remap(O.CLAMP, i, 2, 7) for i in (0, 1, 2, 6, 7, 9)] == [2, 2, 2, 6, 6, 6]
    assert [O.remap(O.REPEAT, i, 2, 7) for i in (0, 1, 7, 8, -9)] == [5, 6, 2, 3, 6]
    assert [O.remap(O.MIRROR, i, 2, 7) for i in (1, 0, 7, 8)] == [2, 3, 6, 5]
    # beyond one reflection the oracle keeps reflecting (definition shared with the kernels)
    assert O.remap(O.MIRROR, -5, 0, 1) == 0 and O.remap(O.MIRROR, -3, 0, 2) == 1
    assert O.remap(O.CONSTANT, -1, 0, 5) == -2147483648


@pytest.mark.parametrize("b", [1, 2, 3])
def test_live_reference_pin(oracle, b):
    """Fresh random inputs against the reference build (only where it exists)."""
    O = oracle
    R = O.ref()
    if R is None:
        pytest.skip("reference tree not present")
    rng = np.random.default_rng(100 + b)
    for (mh, mw) in [(3, 3), (7, 7), (1, 13), (13, 1)]:
        img = rng.random((33, 41), dtype=np.float32)
        m = rng.random((mh, mw)).astype(np.float32)
        r = np.zeros_like(img)
        R.ref_conv_f32(img, 41, 33, m, mw, mh, b, 0, 0, r)
        assert np.array_equal(O.local_op(img, mask=m, boundary=b, contract=0), r)
    img = rng.integers(0, 256, (40, 52), dtype=np.uint8)
    r = np.zeros_like(img)
    R.ref_sobel_mag_u8(img, 52, 40, O.SOBEL3_X, O.SOBEL3_Y, 3, b, r)
    assert np.array_equal(O.sobel_mag(img, boundary=b), r)
    # the separable form: the reference writes it as two DSL convolutions (1x9, then 9x1)
    img = rng.random((31, 43), dtype=np.float32)
    taps = O.gaussian_taps(9, 2.0)
    tmp, r = np.zeros_like(img), np.zeros_like(img)
    assert R.ref_conv_f32(img, 43, 31, np.ascontiguousarray(taps[None, :]), 9, 1, b, 0, 0, tmp) == 0
    assert R.ref_conv_f32(tmp, 43, 31, np.ascontiguousarray(taps[:, None]), 1, 9, b, 0, 0, r) == 0
    assert np.array_equal(O.separable(img, taps, taps, boundary=b, contract=0), r)
    # u8 images through the samples' own uchar kernels (blur with + 0.5f, erode / dilate)
    for (mh, mw) in [(3, 3), (5, 5), (7, 7)]:
        img = rng.integers(0, 256, (29, 37), dtype=np.uint8)
        m = rng.random((mh, mw)).astype(np.float32)
        m /= m.sum()
        r = np.zeros_like(img)
        assert R.ref_conv_u8(img, 37, 29, m, mw, mh, b, 0, 0, r) == 0
        assert np.array_equal(O.local_op_u8(img, mask=m, boundary=b, contract=0), r)
    for red in (O.MIN, O.MAX):
        img = rng.integers(0, 256, (29, 37), dtype=np.uint8)
        dom = (rng.random((5, 5)) > 0.3).astype(np.float32)
        dom[2, 2] = 1.0
        r = np.zeros_like(img)
        assert R.ref_conv_u8(img, 37, 29, dom, 5, 5, b, 1, red, r) == 0
        got = O.local_op_u8(img, domain=dom.astype(np.uint8), size=(5, 5), reduce=red, boundary=b, contract=0)
        assert np.array_equal(got, r), red
    if b != O.CONSTANT:  # the programs' DSL runs honour CLAMP / REPEAT / MIRROR
        img = rng.integers(0, 256, (35, 44), dtype=np.uint8)
        r = np.zeros_like(img)
        R.ref_harris_u8(img, 44, 35, b, 0.04, 20000.0, r)
        assert np.array_equal(O.harris(img, b), r)
        rgba = rng.integers(0, 256, (27, 31, 4), dtype=np.uint8)
        ro = np.zeros_like(rgba)
        R.ref_unsharp_u8x4(rgba.reshape(27, 31 * 4), 31, 27, b, ro.reshape(27, 31 * 4), None)
        assert np.array_equal(O.unsharp(rgba, b)[0], ro)
    f = rng.random((40, 52), dtype=np.float32)
    nc = R.ref_cpu_red_cores_omp()
    assert np.float32(R.ref_cpu_red_sum_f32_omp(f, 52, 40)) == np.float32(O.reduce_f32(f, O.SUM, nc))


def test_harris_unsharp_golden(oracle, golden):
    """The Harris corner and Unsharp sample programs as the reference's DSL ran
    them: bit-exact, luminance included."""
    O = oracle
    for b in (O.CLAMP, O.REPEAT, O.MIRROR):
        assert np.array_equal(O.harris(golden[f"harris_b{b}_in"], b), golden[f"harris_b{b}_out"]), b
        o, g = O.unsharp(golden[f"unsharp_b{b}_in"], b)
        assert np.array_equal(o, golden[f"unsharp_b{b}_out"]), b
        assert np.array_equal(g, golden[f"unsharp_b{b}_gray"]), b


def test_adjoint_oracle_matches_finite_differences(oracle):
    """The FP64 hand adjoint of conv -> bilateral -> MSE against central differences."""
    O = oracle
    rng = np.random.default_rng(7)
    for b in (O.CLAMP, O.MIRROR):
        x = rng.random((10, 12))
        t = rng.random((10, 12))
        mask = rng.normal(0, 0.2, (7, 7))
        sm = O.spatial_mask(9, 2.0, np.float64)
        loss, dx, dm, ds = O.c5_grad(x, t, mask, sm, 0.15, b)
        eps = 1e-5
        for (i, j) in [(0, 0), (9, 11), (4, 5)]:
            xp, xm = x.copy(), x.copy()
            xp[i, j] += eps
            xm[i, j] -= eps
            fd = (O.c5_loss(xp, t, mask, sm, 0.15, b) - O.c5_loss(xm, t, mask, sm, 0.15, b)) / (2 * eps)
            assert abs(fd - dx[i, j]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9
        mp, mm = mask.copy(), mask.copy()
        mp[3, 2] += eps
        mm[3, 2] -= eps
        fd = (O.c5_loss(x, t, mp, sm, 0.15, b) - O.c5_loss(x, t, mm, sm, 0.15, b)) / (2 * eps)
        assert abs(fd - dm[3, 2]) <= 1e-6 * max(1.0, abs(fd))
        fd = (O.c5_loss(x, t, mask, sm, 0.15 + eps, b) - O.c5_loss(x, t, mask, sm, 0.15 - eps, b)) / (2 * eps)
        assert abs(fd - ds) <= 1e-6 * max(1.0, abs(fd))
