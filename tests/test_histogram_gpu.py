"""GPU parity of the histogram binning kernel against the oracle (bit-exact
integer counts): u8 and f32 pixels, several bin counts, windows, batches,
values past the last bin, pitched rows."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _bins(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("hw", [(4096, 4096), (33, 47), (1, 1), (5, 4099)])
@pytest.mark.parametrize("nb", [256, 7, 1000])
def test_histogram_u8(gpu, oracle, hw, nb):
    rng = np.random.default_rng(hw[0] + nb)
    img = rng.integers(0, 256, hw, dtype=np.uint8)
    got = _bins(gpu.histogram(torch.from_numpy(img).cuda(), nb))
    assert np.array_equal(got, oracle.histogram(img, nb))


@pytest.mark.parametrize("nb", [256, 64, 16384])
def test_histogram_f32(gpu, oracle, nb):
    rng = np.random.default_rng(nb)
    img = (rng.random((777, 1031)) * 255.0).astype(np.float32)
    img[0, :4] = [255.0, 0.0, 254.999, -3.0]  # past the last bin, first bin, last bin, negative
    got = _bins(gpu.histogram(torch.from_numpy(img).cuda(), nb))
    assert np.array_equal(got, oracle.histogram(img, nb))


def test_histogram_window_pitched_batch(gpu, oracle):
    rng = np.random.default_rng(3)
    big = rng.integers(0, 256, (3, 70, 96), dtype=np.uint8)
    t = torch.from_numpy(big).cuda()
    # window of every image of the batch
    got = _bins(gpu.histogram(t[:, :, :80], 256, win=(5, 7, 60, 50)))
    ref = sum(oracle.histogram(np.ascontiguousarray(big[b, 7:57, 5:65]), 256).astype(np.int64) for b in range(3))
    assert np.array_equal(got.astype(np.int64), ref)
    # dense batch
    got = _bins(gpu.histogram(t, 100))
    ref = sum(oracle.histogram(big[b], 100).astype(np.int64) for b in range(3))
    assert np.array_equal(got.astype(np.int64), ref)
