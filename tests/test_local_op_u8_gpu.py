"""GPU parity of hgb_local_op on u8 images against the oracle.

Hipacc's own image samples run on `Image<uchar>`: the blur writes
`output() = (uchar)(convolve(mask, Reduce::SUM, ...) + 0.5f)`
(samples-public/1_Local_Operators/Gaussian_Blur/src/main.cpp), erode and
dilate write the MIN / MAX of a domain reduction.  u8 storage reproduces that:
pixels are widened to float, the operator runs in FP32 exactly as for f32
images, and the result is written as (uchar)(v + 0.5f) with values outside
[0, 255] saturated.  The oracle computes the FP32 result on the widened input
and the same write rule is applied here, so the bar is bit-exact.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MODES = [1, 2, 3, 4]  # CLAMP, REPEAT, MIRROR, CONSTANT


def _write_u8(v):
    """(uchar)(v + 0.5f) in FP32, saturated to [0, 255] (the oracle's write rule,
    pinned to the reference's u8 samples in test_oracle_golden.py)."""
    from oracle import write_u8
    return write_u8(v)


def _img(rng, h, w):
    return rng.integers(0, 256, size=(h, w), dtype=np.uint8)


@pytest.mark.parametrize("shape", [(3, 3), (5, 5), (7, 7), (9, 9), (11, 11), (13, 13), (1, 5), (7, 1), (4, 4)])
@pytest.mark.parametrize("b", MODES)
def test_conv_u8_bitexact(gpu, oracle, shape, b):
    rng = np.random.default_rng(hash(("u8", shape, b)) % 2**32)
    mh, mw = shape
    for (h, w) in [(37, 45), (70, 130), (16, 16), (64, 256)]:
        img = _img(rng, h, w)
        m = rng.random((mh, mw)).astype(np.float32)
        m /= m.sum()
        t = torch.from_numpy(img).cuda()
        out = torch.zeros_like(t)
        gpu.local_op(t, out, mask=m, boundary=b, const=17.0)
        ref = _write_u8(oracle.local_op(img.astype(np.float32), mask=m, boundary=b, const=17.0, contract=1))
        got = out.cpu().numpy()
        assert np.array_equal(got, ref), (shape, b, h, w, int(np.abs(got.astype(int) - ref).max()))


def test_gaussian_u8_sample(gpu, oracle):
    """The Gaussian-blur sample's configuration: 5x5 sigma=1 mask, CLAMP, u8 in and out."""
    rng = np.random.default_rng(11)
    img = _img(rng, 1024, 1024)
    m = oracle.gaussian_mask(5, 1.0)
    t = torch.from_numpy(img).cuda()
    out = torch.empty_like(t)
    gpu.local_op(t, out, mask=m, boundary=1)
    ref = _write_u8(oracle.local_op(img.astype(np.float32), mask=m, boundary=1, contract=1))
    assert np.array_equal(out.cpu().numpy(), ref)


def test_saturation(gpu, oracle):
    """A Laplacian-style mask leaves [0, 255]: results saturate at both ends."""
    rng = np.random.default_rng(12)
    img = _img(rng, 48, 80)
    m = np.array([[0, -1, 0], [-1, 4, -1], [0, -1, 0]], np.float32) * 3
    t = torch.from_numpy(img).cuda()
    out = torch.empty_like(t)
    gpu.local_op(t, out, mask=m, boundary=3)
    ref_f = oracle.local_op(img.astype(np.float32), mask=m, boundary=3, contract=1)
    assert (ref_f < 0).any() and (ref_f > 255).any()
    assert np.array_equal(out.cpu().numpy(), _write_u8(ref_f))


@pytest.mark.parametrize("red", [1, 2])
def test_erode_dilate(gpu, oracle, red):
    """Erode / dilate: MIN / MAX over a domain, u8 in and out (general kernel)."""
    rng = np.random.default_rng(13 + red)
    img = _img(rng, 41, 67)
    dom = np.ones((3, 3), np.uint8)
    dom[0, 0] = dom[2, 2] = 0
    t = torch.from_numpy(img).cuda()
    for b in MODES:
        out = torch.empty_like(t)
        gpu.local_op(t, out, domain=dom, size=(3, 3), reduce=red, boundary=b, const=200.0)
        ref = oracle.local_op(img.astype(np.float32), domain=dom, size=(3, 3), reduce=red, boundary=b, const=200.0,
                              contract=1)
        assert np.array_equal(out.cpu().numpy(), _write_u8(ref)), b


def test_u8_to_f32(gpu, oracle):
    """u8 input, FP32 output: the unrounded FP32 result."""
    rng = np.random.default_rng(15)
    img = _img(rng, 33, 50)
    m = oracle.gaussian_mask(7, 1.5)
    t = torch.from_numpy(img).cuda()
    out = torch.empty(img.shape, dtype=torch.float32, device="cuda")
    gpu.local_op(t, out, mask=m, boundary=2)
    ref = oracle.local_op(img.astype(np.float32), mask=m, boundary=2, contract=1)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_u8_windows_and_batch(gpu, oracle):
    """Unaligned accessor / iteration-space offsets and a pitched batch of u8 images."""
    rng = np.random.default_rng(16)
    B, h, w = 3, 45, 99
    imgs = np.stack([_img(rng, h, w) for _ in range(B)])
    big = torch.zeros((B, h, 128), dtype=torch.uint8, device="cuda")
    big[:, :, :w] = torch.from_numpy(imgs).cuda()
    src = big[:, :, :w]
    out = torch.zeros((B, h, 128), dtype=torch.uint8, device="cuda")[:, :, :w]
    m = oracle.gaussian_mask(5, 1.0)
    gpu.local_op(src, out, mask=m, boundary=3)
    got = out.cpu().numpy()
    for i in range(B):
        assert np.array_equal(got[i], _write_u8(oracle.local_op(imgs[i].astype(np.float32), mask=m, boundary=3,
                                                                contract=1)))
    img = imgs[0]
    for b in MODES:
        acc, isp = (13, 5, 50, 30), (7, 3, 50, 30)
        o = torch.zeros((40, 70), dtype=torch.uint8, device="cuda")
        gpu.local_op(torch.from_numpy(img).cuda(), o, mask=m, boundary=b, const=9.0, acc=acc, iter_space=isp)
        ref_f = oracle.local_op(img.astype(np.float32), mask=m, boundary=b, const=9.0, contract=1, acc=acc,
                                out=np.zeros((40, 70), np.float32), iter_space=isp)
        ref = _write_u8(ref_f)
        got = o.cpu().numpy()
        inside = np.zeros((40, 70), bool)
        inside[3:33, 7:57] = True
        assert np.array_equal(got[inside], ref[inside]), b
        assert not got[~inside].any()
