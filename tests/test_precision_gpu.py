"""GPU parity of the separable and bilateral filters across storage types.

Separable: bit-exact against the oracle's two-pass FP32 program (1xK then Kx1
local operators with an FP32 intermediate image), contracted form.  BF16 /
F16 storage: the oracle runs on the widened input and its FP32 result is
rounded to nearest even -- the kernel keeps the intermediate in FP32, so this
is bit-exact too.

Bilateral: FP32 within BIL_F32_TOL of the oracle's FP32 form (the kernel's
exp2 instruction and folded spatial weight differ from libm's expf by a few
ulp); every storage type within 1e-2 relative of the FP64 oracle, the bar for
reduced-precision forms.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

BIL_F32_TOL = 2e-5  # max |gpu - oracle_f32| / max(|oracle_f32|, 1e-3)
REDUCED_TOL = 1e-2  # max relative error against FP64 for BF16/F16 storage


def field(h, w, seed):
    """Smooth 2-D sinusoid plus N(0, 0.05) noise, clipped to [0, 1]."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    f = 0.5 + 0.25 * np.sin(2 * np.pi * x / 512.0) * np.cos(2 * np.pi * y / 384.0) + rng.normal(0, 0.05, (h, w))
    return np.clip(f, 0.0, 1.0).astype(np.float32)


def _sep(api, img, taps, b, const, dtype=torch.float32):
    t = torch.from_numpy(img).to(dtype).cuda()
    out = torch.empty_like(t)
    api.separable(t, out, taps, taps, boundary=b, const=const)
    torch.cuda.synchronize()
    return out.cpu()


@pytest.mark.parametrize("k", [3, 5, 9, 15])
@pytest.mark.parametrize("b", [1, 2, 3, 4])
def test_separable_f32_bitexact(gpu, oracle, k, b):
    rng = np.random.default_rng(k * 10 + b)
    for (h, w) in [(45, 131), (64, 128), (7, 300)]:
        img = rng.random((h, w), dtype=np.float32)
        taps = oracle.gaussian_taps(k, 2.0)
        got = _sep(gpu, img, taps, b, 0.5).numpy()
        ref = oracle.separable(img, taps, taps, boundary=b, const=0.5, contract=1)
        assert np.array_equal(got, ref), (k, b, h, w, np.abs(got - ref).max())


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("b", [2, 4])
def test_separable_half_storage(gpu, oracle, dtype, b):
    img = field(70, 200, 3)
    src = torch.from_numpy(img).to(dtype)
    taps = oracle.gaussian_taps(9, 2.0)
    got = _sep(gpu, src.float().numpy(), taps, b, 0.5, dtype)
    ref = torch.from_numpy(oracle.separable(src.float().numpy(), taps, taps, boundary=b, const=0.5)).to(dtype)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16, torch.float16])
@pytest.mark.parametrize("b", [1, 2, 3, 4])
def test_separable_many_tiles(gpu, oracle, dtype, b):
    """A multi-tile image with ragged edges and unpadded rows of 1301 elements,
    which no storage type aligns to 16 bytes, so the tiles are staged with
    plain loads instead of TMA: bit-exact in every storage type."""
    img = field(517, 1301, 7 + b)
    src = torch.from_numpy(img).to(dtype)
    taps = oracle.gaussian_taps(9, 2.0)
    got = _sep(gpu, src.float().numpy(), taps, b, 0.5, dtype)
    ref = torch.from_numpy(oracle.separable(src.float().numpy(), taps, taps, boundary=b, const=0.5,
                                            contract=1)).to(dtype)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("k", [3, 5, 7, 9, 11, 13, 15])
def test_separable_tma_half_storage(gpu, oracle, dtype, k):
    """16-bit storage with rows padded to 16 bytes takes the TMA-staged form:
    bit-exact for every mask size, every boundary, ragged and odd widths,
    images shorter than the mask, several tiles in both directions, and a
    batch."""
    rng = np.random.default_rng(100 + k)
    taps = oracle.gaussian_taps(k, 2.0)
    cases = [((517, 1301), 1, 1), ((300, 130), 2, 1), ((1, 9), 3, 1), ((5, 3), 4, 1), ((257, 129), 3, 2),
             ((600, 256), 4, 1), ((33, 700), 2, 3)]
    for (h, w), b, nb in cases:
        img = field(h, w * nb, k + b)[:, :w * nb].reshape(h, nb, w).transpose(1, 0, 2).copy()
        img = np.clip(img + rng.normal(0, 0.01, img.shape).astype(np.float32), 0, 1)
        src = torch.from_numpy(img).to(dtype)
        wp = (w + 7) // 8 * 8 + 8
        dev = torch.zeros((nb, h, wp), dtype=dtype, device="cuda")
        dev[:, :, :w] = src.cuda()
        out = torch.full((nb, h, wp), 3.0, dtype=dtype, device="cuda")
        s_in, s_out = (dev[:, :, :w], out[:, :, :w]) if nb > 1 else (dev[0, :, :w], out[0, :, :w])
        gpu.separable(s_in, s_out, taps, taps, boundary=b, const=0.5)
        torch.cuda.synchronize()
        got = out.cpu()
        for i in range(nb):
            ref = torch.from_numpy(oracle.separable(src[i].float().numpy(), taps, taps, boundary=b, const=0.5,
                                                    contract=1)).to(dtype)
            assert torch.equal(got[i, :, :w], ref), (k, h, w, b, i)
            assert torch.all(got[i, :, w:] == 3.0)  # nothing written past the width


@pytest.mark.parametrize("b", [2, 4])
def test_separable_8192(gpu, oracle, b):
    """The 9x9 sigma=2 separable Gaussian on the 8192x8192 field, REPEAT and CONSTANT(0.5)."""
    img = field(8192, 8192, 11)
    taps = oracle.gaussian_taps(9, 2.0)
    got = _sep(gpu, img, taps, b, 0.5).numpy()
    assert np.array_equal(got, oracle.separable(img, taps, taps, boundary=b, const=0.5, contract=1))
    # reduced-precision storage against FP64
    ref64 = oracle.separable(img[:1024, :1024].astype(np.float64), taps.astype(np.float64), taps.astype(np.float64),
                             boundary=b, const=0.5)
    for dtype in (torch.bfloat16, torch.float16):
        g = _sep(gpu, img[:1024, :1024].copy(), taps, b, 0.5, dtype).double().numpy()
        rel = np.max(np.abs(g - ref64) / np.maximum(np.abs(ref64), 1e-3))
        assert rel <= REDUCED_TOL, (dtype, rel)


def _bil(api, img, sm, sigma, b, const, dtype=torch.float32, fast=False):
    t = torch.from_numpy(img).to(dtype).cuda()
    out = torch.empty_like(t)
    api.bilateral(t, out, sm, sigma, boundary=b, const=const, fast_weights=fast)
    torch.cuda.synchronize()
    return out.cpu()


@pytest.mark.parametrize("size", [3, 5, 9, 13])
@pytest.mark.parametrize("b", [1, 2, 3, 4])
def test_bilateral_f32(gpu, oracle, size, b):
    img = field(61, 150, size + b)
    sm = oracle.spatial_mask(size, 3.0)
    got = _bil(gpu, img, sm, 0.1, b, 0.5).numpy()
    ref = oracle.bilateral(img, sm, 0.1, boundary=b, const=0.5)
    err = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3))
    assert err <= BIL_F32_TOL, err


def test_bilateral_zero_weights_are_skipped(gpu, oracle):
    """Domain(mask) semantics: zero spatial weights contribute nothing."""
    img = field(40, 70, 5)
    sm = oracle.spatial_mask(5, 2.0)
    sm[0, :] = 0.0
    sm[:, 4] = 0.0
    got = _bil(gpu, img, sm, 0.2, 3, 0.0).numpy()
    ref = oracle.bilateral(img, sm, 0.2, boundary=3)
    assert np.max(np.abs(got - ref)) <= BIL_F32_TOL


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("fast", [False, True])
def test_bilateral_reduced_precision(gpu, oracle, dtype, fast):
    """13x13 sigma_d=3, sigma_r=0.1 bilateral on BF16 / F16 storage vs FP64."""
    img = field(256, 384, 9)
    stored = torch.from_numpy(img).to(dtype).float().numpy()
    sm = oracle.spatial_mask(13, 3.0)
    for b in (2, 4):
        got = _bil(gpu, stored, sm, 0.1, b, 0.5, dtype, fast).double().numpy()
        ref = oracle.bilateral(stored.astype(np.float64), sm.astype(np.float64), 0.1, boundary=b, const=0.5)
        rel = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3))
        assert rel <= REDUCED_TOL, (dtype, fast, b, rel)


def test_bilateral_8192_f32(gpu, oracle):
    """The 13x13 bilateral on the 8192x8192 field (REPEAT), checked on row bands."""
    img = field(8192, 8192, 13)
    sm = oracle.spatial_mask(13, 3.0)
    got = _bil(gpu, img, sm, 0.1, 2, 0.0).numpy()
    ref = oracle.bilateral(img, sm, 0.1, boundary=2)
    err = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3))
    assert err <= BIL_F32_TOL, err
