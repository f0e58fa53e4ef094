"""CPU: the oracle's FP64 hand adjoint of the bilateral filter against FP64
central differences of the oracle's FP64 forward (the bilateral body of
samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77), every
boundary mode; this pins the restatement the GPU adjoint is checked against."""
import numpy as np
import pytest


@pytest.mark.parametrize("boundary,const", [(1, 0.0), (2, 0.0), (3, 0.0), (4, 0.3)])
def test_bilateral_adjoint_oracle_vs_central_differences(oracle, boundary, const):
    rng = np.random.default_rng(boundary)
    x = rng.random((21, 17))
    g = rng.normal(0, 1, (21, 17))
    sm = oracle.spatial_mask(5, 1.2).astype(np.float64)
    sigma = 0.15
    gi, gs = oracle.bilateral_adjoint(x, g, sm, sigma, boundary, const)
    f = lambda xx, s: float(np.sum(g * oracle.bilateral(xx, sm, s, boundary, const)))
    eps = 1e-5
    for (i, j) in [(0, 0), (20, 16), (0, 8), (10, 0), (1, 15), (10, 8)]:
        xp, xm = x.copy(), x.copy()
        xp[i, j] += eps
        xm[i, j] -= eps
        fd = (f(xp, sigma) - f(xm, sigma)) / (2 * eps)
        assert abs(gi[i, j] - fd) <= 1e-6 * max(abs(fd), 1.0), (i, j, gi[i, j], fd)
    fd = (f(x, sigma + eps) - f(x, sigma - eps)) / (2 * eps)
    assert abs(gs - fd) <= 1e-6 * max(abs(fd), 1.0)


@pytest.mark.parametrize("boundary", [0, 1, 2, 3, 4])
def test_separable_adjoint_oracle_is_the_transpose(oracle, boundary):
    """<sep(x), y> = <x, sep^T(y)> with the oracle's FP64 forward, and the tap
    gradients equal the exact change of <sep(x), y> per unit tap (the forward
    is linear in each tap vector).  CONSTANT with constant 0, where the forward
    is linear."""
    rng = np.random.default_rng(30 + boundary)
    x = rng.random((19, 23))
    y = rng.normal(0, 1, (19, 23))
    row, col = rng.normal(0, 1, 5), rng.normal(0, 1, 5)
    f = lambda r, c: float(np.sum(y * oracle.separable(x, r, c, boundary=boundary, const=0.0, contract=0)))
    gin, grow, gcol = oracle.separable_adjoint(x, y, row, col, boundary, 0.0)
    assert abs(f(row, col) - float(np.sum(x * gin))) <= 1e-10 * max(abs(f(row, col)), 1.0)
    for j in range(5):
        e = np.zeros(5)
        e[j] = 1.0
        assert abs((f(row + e, col) - f(row, col)) - grow[j]) <= 1e-9 * max(abs(grow[j]), 1.0)
        assert abs((f(row, col + e) - f(row, col)) - gcol[j]) <= 1e-9 * max(abs(gcol[j]), 1.0)


@pytest.mark.parametrize("reduce", [1, 2])
@pytest.mark.parametrize("boundary", [0, 1, 2, 3, 4])
def test_minmax_oracle_forward_is_the_reference(oracle, reduce, boundary):
    """The MIN / MAX rule the adjoint follows gives the reference's own values:
    the oracle's local_op (pinned to the reference by the golden vectors) for a
    Domain and for a mask, ties and FLT_MIN / FLT_MAX start values included."""
    rng = np.random.default_rng(40 + 10 * reduce + boundary)
    dom = (rng.random((5, 5)) < 0.6).astype(np.uint8)
    dom[2, 2] = 1
    mask = rng.normal(0, 1, (3, 3)).astype(np.float32)
    for img in (rng.random((17, 23)).astype(np.float32) - 0.25, rng.integers(0, 3, (17, 23)).astype(np.float32)):
        out, _ = oracle.minmax_adjoint(img, np.zeros_like(img), reduce, domain=dom, boundary=boundary, const=0.125)
        ref = oracle.local_op(img, domain=dom, reduce=reduce, boundary=boundary, const=0.125)
        assert np.array_equal(out, ref)
        out, _ = oracle.minmax_adjoint(img, np.zeros_like(img), reduce, mask=mask, boundary=boundary, const=0.125)
        ref = oracle.local_op(img, mask=mask, reduce=reduce, boundary=boundary, const=0.125)
        assert np.array_equal(out, ref)


def test_minmax_adjoint_oracle_vs_loops(oracle):
    """The vectorised MIN / MAX adjoint against plain loops over outputs and taps."""
    rng = np.random.default_rng(77)
    h, w = 9, 11
    img = rng.integers(0, 3, (h, w)).astype(np.float32)
    g = rng.normal(0, 1, (h, w))
    dom = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], np.uint8)
    for reduce, boundary in ((1, 1), (2, 2), (2, 3), (1, 4), (2, 0)):
        _, gin = oracle.minmax_adjoint(img, g, reduce, domain=dom, boundary=boundary, const=1.0)
        ref = np.zeros((h, w))
        for yy in range(h):
            for xx in range(w):
                acc = np.float32(np.finfo(np.float32).tiny if reduce == 2 else np.finfo(np.float32).max)
                src = None
                for my in range(3):
                    for mx in range(3):
                        if not dom[my, mx]:
                            continue
                        ry, rx = oracle.remap(boundary, yy + my - 1, 0, h), oracle.remap(boundary, xx + mx - 1, 0, w)
                        outside = ry < 0 or rx < 0
                        v = np.float32(1.0) if outside else img[ry, rx]
                        if not ((acc > v) if reduce == 2 else (acc < v)):
                            acc, src = v, None if outside else (ry, rx)
                if src is not None:
                    ref[src] += g[yy, xx]
        assert np.allclose(gin, ref, rtol=0, atol=1e-12), (reduce, boundary)
