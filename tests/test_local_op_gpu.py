"""GPU parity of hgb_local_op against the oracle.

Bar: bit-exact against the FMA-contracted oracle (the kernels accumulate
row-major with fused multiply-add, as the contracted reference code does) and
within 1e-6 relative of the separately rounded reference form.  BF16 / F16
storage: the oracle runs on the widened input and its FP32 result is rounded
to nearest even, which the kernels must match bit for bit.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MODES = [1, 2, 3, 4]  # CLAMP, REPEAT, MIRROR, CONSTANT
REL_TOL = 1e-6  # against the uncontracted reference form


def _run(api, img, mask=None, domain=None, size=None, reduce=0, boundary=1, const=0.0, acc=None, iter_space=None,
         out_shape=None, dtype=torch.float32):
    t = torch.from_numpy(img).cuda().to(dtype)
    out = torch.zeros(out_shape or img.shape, dtype=dtype, device="cuda")
    api.local_op(t, out, mask=mask, domain=domain, size=size, reduce=reduce, boundary=boundary, const=const, acc=acc,
                 iter_space=iter_space)
    torch.cuda.synchronize()
    return out.float().cpu().numpy()


@pytest.mark.parametrize("shape", [(3, 3), (5, 5), (7, 7), (9, 9), (13, 13), (1, 9), (9, 1), (1, 3), (13, 1),
                                   (4, 4), (3, 5), (2, 6)])
@pytest.mark.parametrize("b", MODES)
def test_conv_f32_bitexact(gpu, oracle, shape, b):
    rng = np.random.default_rng(hash((shape, b)) % 2**32)
    mh, mw = shape
    for (h, w) in [(37, 45), (70, 130), (16, 16)]:
        img = rng.random((h, w), dtype=np.float32)
        m = rng.random((mh, mw)).astype(np.float32)
        got = _run(gpu, img, mask=m, boundary=b, const=0.5)
        ref_fma = oracle.local_op(img, mask=m, boundary=b, const=0.5, contract=1)
        assert np.array_equal(got, ref_fma), (shape, b, h, w, np.abs(got - ref_fma).max())
        ref = oracle.local_op(img, mask=m, boundary=b, const=0.5, contract=0)
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)) <= REL_TOL


def test_gaussian_1024_clamp(gpu, oracle):
    """The 5x5 sigma=1 Gaussian on 1024x1024 FP32 with CLAMP."""
    rng = np.random.default_rng(1)
    img = rng.random((1024, 1024), dtype=np.float32)
    m = oracle.gaussian_mask(5, 1.0)
    got = _run(gpu, img, mask=m, boundary=1)
    assert np.array_equal(got, oracle.local_op(img, mask=m, boundary=1, contract=1))
    ref = oracle.local_op(img, mask=m, boundary=1, contract=0)
    assert np.max(np.abs(got - ref) / ref) <= REL_TOL


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("b", [1, 3, 4])
def test_conv_half_storage(gpu, oracle, dtype, b):
    rng = np.random.default_rng(3)
    img = rng.random((67, 129), dtype=np.float32)
    src = torch.from_numpy(img).to(dtype)
    widened = src.float().numpy()
    m = oracle.gaussian_mask(7, 1.5)
    t = src.cuda()
    out = torch.zeros_like(t)
    gpu.local_op(t, out, mask=m, boundary=b, const=0.5)
    ref = torch.from_numpy(oracle.local_op(widened, mask=m, boundary=b, const=0.5, contract=1)).to(dtype)
    assert torch.equal(out.cpu(), ref)


def test_batch_and_pitch(gpu, oracle):
    """A batch of images in one launch, rows padded (pitch > width)."""
    rng = np.random.default_rng(4)
    B, h, w = 5, 50, 77
    imgs = rng.random((B, h, w), dtype=np.float32)
    big = torch.zeros((B, h, 96), device="cuda")
    big[:, :, :w] = torch.from_numpy(imgs).cuda()
    src = big[:, :, :w]
    out = torch.zeros((B, h, 96), device="cuda")[:, :, :w]
    m = oracle.gaussian_mask(5, 1.0)
    gpu.local_op(src, out, mask=m, boundary=3)
    got = out.cpu().numpy()
    for i in range(B):
        assert np.array_equal(got[i], oracle.local_op(imgs[i], mask=m, boundary=3, contract=1))


def test_roi_windows(gpu, oracle):
    """Accessor window and IterationSpace offsets (boundary relative to the window)."""
    rng = np.random.default_rng(5)
    img = rng.random((60, 90), dtype=np.float32)
    m = rng.random((5, 5)).astype(np.float32)
    for b in MODES:
        acc = (12, 7, 40, 30)
        out = np.zeros((50, 70), np.float32)
        ref = oracle.local_op(img, mask=m, boundary=b, const=0.25, contract=1, acc=acc, out=out.copy(),
                              iter_space=(20, 9, 40, 30))
        got = _run(gpu, img, mask=m, boundary=b, const=0.25, acc=acc, iter_space=(20, 9, 40, 30),
                   out_shape=(50, 70))
        assert np.array_equal(got, ref), b


@pytest.mark.parametrize("red", [1, 2, 3])
def test_domain_reduce_generic(gpu, oracle, red):
    """Kernel::reduce(Domain, MIN/MAX/PROD) through the general kernel."""
    rng = np.random.default_rng(6 + red)
    img = (rng.random((41, 53), dtype=np.float32) + 0.5).astype(np.float32)
    dom = (rng.random((5, 5)) > 0.4).astype(np.uint8)
    dom[2, 2] = 1
    for b in MODES:
        got = _run(gpu, img, domain=dom, size=(5, 5), reduce=red, boundary=b, const=0.75)
        ref = oracle.local_op(img, domain=dom, size=(5, 5), reduce=red, boundary=b, const=0.75, contract=1)
        if red == 3:
            np.testing.assert_allclose(got, ref, rtol=1e-5)
        else:
            assert np.array_equal(got, ref)


def test_max_init_is_flt_min(gpu, oracle):
    """Compiled MAX starts at numeric_limits<float>::min() (lib/AST/Convolution.cpp:90-100)."""
    img = -np.ones((20, 20), np.float32)
    dom = np.ones((3, 3), np.uint8)
    got = _run(gpu, img, domain=dom, size=(3, 3), reduce=2, boundary=1)
    assert np.all(got == np.float32(1.17549435e-38))
    assert np.array_equal(got, oracle.local_op(img, domain=dom, size=(3, 3), reduce=2, boundary=1))


def test_sum_domain_and_mask_domain(gpu, oracle):
    rng = np.random.default_rng(8)
    img = rng.random((33, 47), dtype=np.float32)
    dom = (rng.random((3, 3)) > 0.3).astype(np.uint8)
    got = _run(gpu, img, domain=dom, size=(3, 3), boundary=3)
    assert np.array_equal(got, oracle.local_op(img, domain=dom, size=(3, 3), boundary=3, contract=1))
    m = rng.random((3, 3)).astype(np.float32)
    got = _run(gpu, img, mask=m, domain=dom, boundary=2)
    assert np.array_equal(got, oracle.local_op(img, mask=m, domain=dom, boundary=2, contract=1))


def test_large_and_device_mask(gpu, oracle):
    """15x15 masks and device-resident masks take the general kernel."""
    rng = np.random.default_rng(9)
    img = rng.random((40, 44), dtype=np.float32)
    m = rng.random((15, 15)).astype(np.float32)
    got = _run(gpu, img, mask=m, boundary=3)
    assert np.array_equal(got, oracle.local_op(img, mask=m, boundary=3, contract=1))
    m7 = rng.random((7, 7)).astype(np.float32)
    t = torch.from_numpy(img).cuda()
    out = torch.empty_like(t)
    gpu.local_op(t, out, mask_dev=torch.from_numpy(m7).cuda(), size=(7, 7), boundary=1)
    assert np.array_equal(out.cpu().numpy(), oracle.local_op(img, mask=m7, boundary=1, contract=1))


@pytest.mark.parametrize("hw", [(1, 1), (1, 37), (37, 1), (2, 3), (3, 2), (257, 5), (5, 4095)])
def test_odd_sizes(gpu, oracle, hw):
    """Tiny and ragged images; MIRROR with a radius beyond the image iterates the reflection."""
    rng = np.random.default_rng(sum(hw))
    img = rng.random(hw, dtype=np.float32)
    m = rng.random((5, 5)).astype(np.float32)
    for b in MODES:
        got = _run(gpu, img, mask=m, boundary=b, const=0.5)
        assert np.array_equal(got, oracle.local_op(img, mask=m, boundary=b, const=0.5, contract=1)), (hw, b)


def test_undefined_interior(gpu, oracle):
    """UNDEFINED: only pixels whose taps stay inside are defined by the reference."""
    rng = np.random.default_rng(10)
    img = rng.random((30, 40), dtype=np.float32)
    m = rng.random((5, 5)).astype(np.float32)
    got = _run(gpu, img, mask=m, boundary=0)
    ref = oracle.local_op(img, mask=m, boundary=0, contract=1)
    assert np.array_equal(got[2:-2, 2:-2], ref[2:-2, 2:-2])


def test_autotune_consistency(gpu, oracle, tmp_path):
    """Every tile configuration gives identical results; choices persist as JSON."""
    from hipacc_gb300 import _lib as L

    rng = np.random.default_rng(11)
    img = rng.random((300, 260), dtype=np.float32)
    m = oracle.gaussian_mask(9, 2.0)
    ref = oracle.local_op(img, mask=m, boundary=2, contract=1)
    L.call("hgb_autotune_clear")
    gpu.autotune(True)
    try:
        got = _run(gpu, img, mask=m, boundary=2)
        assert np.array_equal(got, ref)
        assert L.load().hgb_autotune_count() >= 1
        path = str(tmp_path / "tune.json")
        L.call("hgb_autotune_save", path.encode())
        L.call("hgb_autotune_clear")
        L.call("hgb_autotune_load", path.encode())
        assert L.load().hgb_autotune_count() >= 1
        assert np.array_equal(_run(gpu, img, mask=m, boundary=2), ref)
    finally:
        gpu.autotune(False)
        L.call("hgb_autotune_clear")
