"""GPU parity of the two multi-kernel sample programs built as fused chains:
Harris corner (samples-public/3_Preprocessing/Harris_Corner, 3x3) and Unsharp
(samples-public/1_Local_Operators/Unsharp, 3x3), each in the fused form
(mode 0) and in the reference's launch structure (mode 1: nine and five
launches).  Bar: bit-exact against the oracle, whose programs are pinned to the
reference's own DSL run (golden arrays, test_oracle_golden.py), at the
samples' 4032 x 3024 size, on ragged sizes, pitched batches and every
boundary mode."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def blocks_u8(rng, h, w, n=40, noise=6):
    """Random rectangles of random grey levels plus noise (corners, edges, flat regions)."""
    img = np.full((h, w), int(rng.integers(0, 256)), np.int32)
    for _ in range(n):
        y0, x0 = int(rng.integers(0, max(1, h - 2))), int(rng.integers(0, max(1, w - 2)))
        y1, x1 = int(rng.integers(y0 + 1, h + 1)), int(rng.integers(x0 + 1, w + 1))
        img[y0:y1, x0:x1] = int(rng.integers(0, 256))
    img += rng.integers(-noise, noise + 1, (h, w))
    return np.clip(img, 0, 255).astype(np.uint8)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("b", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("hw", [(37, 53), (130, 257), (1, 1), (2, 9), (300, 64)])
def test_harris_bitexact(gpu, oracle, mode, b, hw):
    rng = np.random.default_rng(hash((mode, b, hw)) % 2**32)
    img = blocks_u8(rng, *hw)
    out = gpu.harris(torch.from_numpy(img).cuda(), boundary=b, mode=mode)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.harris(img, b))


@pytest.mark.parametrize("mode", [0, 1])
def test_harris_sample_size_and_batch(gpu, oracle, mode):
    rng = np.random.default_rng(11 + mode)
    img = blocks_u8(rng, 3024, 4032, n=400)
    out = gpu.harris(torch.from_numpy(img).cuda(), mode=mode)
    torch.cuda.synchronize()
    ref = oracle.harris(img, 1)
    assert np.array_equal(out.cpu().numpy(), ref)
    assert 0 < int(ref.sum()) < ref.size // 2  # corners and non-corners both present
    # a batch of three pitched images, k and threshold varied
    imgs = np.stack([blocks_u8(rng, 201, 333) for _ in range(3)])
    dev = torch.zeros((3, 201, 352), dtype=torch.uint8, device="cuda")
    dev[:, :, :333] = torch.from_numpy(imgs).cuda()
    o = torch.full((3, 201, 352), 9, dtype=torch.uint8, device="cuda")
    gpu.harris(dev[:, :, :333], o[:, :, :333], k=0.06, threshold=5000.0, boundary=3, mode=mode)
    torch.cuda.synchronize()
    got = o.cpu().numpy()
    for i in range(3):
        assert np.array_equal(got[i, :, :333], oracle.harris(imgs[i], 3, k=0.06, threshold=5000.0))
    assert np.all(got[:, :, 333:] == 9)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("b", [1, 2, 3, 4])
@pytest.mark.parametrize("hw", [(33, 47), (129, 200), (1, 1), (5, 3)])
def test_unsharp_bitexact(gpu, oracle, mode, b, hw):
    rng = np.random.default_rng(hash(("u", mode, b, hw)) % 2**32)
    rgba = np.stack([blocks_u8(rng, *hw) for _ in range(4)], axis=-1)
    out = gpu.unsharp(torch.from_numpy(rgba).cuda(), boundary=b, mode=mode)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.unsharp(rgba, b)[0])


@pytest.mark.parametrize("mode", [0, 1])
def test_unsharp_sample_size_and_batch(gpu, oracle, mode):
    """Uniform random channels (every byte value, large ratios whose channel
    products leave [0, 256)) at the samples' size, then a pitched batch."""
    rng = np.random.default_rng(21 + mode)
    rgba = rng.integers(0, 256, (3024, 4032, 4), dtype=np.uint8)
    out = gpu.unsharp(torch.from_numpy(rgba).cuda(), mode=mode)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.unsharp(rgba, 1)[0])
    imgs = rng.integers(0, 256, (2, 77, 90, 4), dtype=np.uint8)
    dev = torch.zeros((2, 77, 96, 4), dtype=torch.uint8, device="cuda")
    dev[:, :, :90] = torch.from_numpy(imgs).cuda()
    o = torch.zeros_like(dev)
    gpu.unsharp(dev[:, :, :90], o[:, :, :90], boundary=3, mode=mode)
    torch.cuda.synchronize()
    got = o.cpu().numpy()
    for i in range(2):
        assert np.array_equal(got[i, :, :90], oracle.unsharp(imgs[i], 3)[0])


def test_pipeline_argument_errors(gpu):
    from hipacc_gb300 import _lib as L

    x = torch.zeros((8, 8), dtype=torch.uint8, device="cuda")
    with pytest.raises(L.HgbError):
        gpu.harris(x, mode=2)
    with pytest.raises(L.HgbError):
        gpu.harris(x, torch.zeros((8, 9), dtype=torch.uint8, device="cuda"))
    c = torch.zeros((8, 8, 4), dtype=torch.uint8, device="cuda")
    with pytest.raises(L.HgbError):
        gpu.unsharp(c, c)
    with pytest.raises(L.HgbError):
        gpu.unsharp(c, boundary=7)
