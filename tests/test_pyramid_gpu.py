"""GPU parity of the batched Laplacian pyramid against the oracle.

All three launch forms (one persistent launch over a work-list of every level
of every image; one launch per level; the reference's per-image per-level
blur / subsample / difference launches) must give the oracle's pyramid bit for
bit (blur taps row-major with fused multiply-add; nearest-neighbour and linear
filtering mappings in FP32 with the contracted mapping), and the collapse must
restore the input (Restore, samples-public/5_Other/Gaussian_Laplacian_Pyramid).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZES = [(257, 300), (300, 257), (513, 129), (97, 1001), (64, 64), (130, 66)]


def _plan(api, oracle, sizes, levels, boundary, seed):
    rng = np.random.default_rng(seed)
    imgs = [rng.random((h, w), dtype=np.float32) for (w, h) in sizes]
    plan = api.PyramidPlan([w for w, _ in sizes], [h for _, h in sizes], levels, oracle.binomial5(), boundary)
    for i, im in enumerate(imgs):
        plan.gauss(i, 0).copy_(torch.from_numpy(im).cuda())
    return plan, imgs


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_pyramid_bitexact(gpu, oracle, mode):
    levels = 6
    plan, imgs = _plan(gpu, oracle, SIZES, levels, oracle.MIRROR, 1)
    plan.decompose(mode)
    torch.cuda.synchronize()
    for i, im in enumerate(imgs):
        g, lap = oracle.pyramid_decompose(im, levels, oracle.binomial5(), oracle.MIRROR, contract=1)
        for l in range(levels):
            assert np.array_equal(plan.gauss(i, l).cpu().numpy(), g[l]), (mode, i, l)
            if l + 1 < levels:
                assert np.array_equal(plan.lap(i, l).cpu().numpy(), lap[l]), (mode, i, l)
    plan.close()


def test_pyramid_persistent_many_images_and_collapse(gpu, oracle):
    """A longer work-list (24 images) through the persistent launch, then the
    collapse restores every input."""
    rng = np.random.default_rng(5)
    sizes = [(int(rng.integers(64, 600)), int(rng.integers(64, 600))) for _ in range(24)]
    levels = 6
    plan, imgs = _plan(gpu, oracle, sizes, levels, oracle.MIRROR, 2)
    plan.decompose(0)
    torch.cuda.synchronize()
    g0 = []
    for i, im in enumerate(imgs):
        g, lap = oracle.pyramid_decompose(im, levels, oracle.binomial5(), oracle.MIRROR, contract=1)
        assert np.array_equal(plan.gauss(i, levels - 1).cpu().numpy(), g[-1])
        assert np.array_equal(plan.lap(i, 0).cpu().numpy(), lap[0])
        g0.append(oracle.pyramid_collapse(g[-1], lap, contract=1)[0])
    plan.collapse()
    torch.cuda.synchronize()
    for i, im in enumerate(imgs):
        r = plan.gauss(i, 0).cpu().numpy()
        assert np.array_equal(r, g0[i])
        assert np.max(np.abs(r - im)) < 1e-5
    plan.close()


@pytest.mark.parametrize("boundary", [1, 2])
def test_pyramid_other_boundaries(gpu, oracle, boundary):
    levels = 5
    plan, imgs = _plan(gpu, oracle, SIZES[:3], levels, boundary, 3)
    plan.decompose(0)
    torch.cuda.synchronize()
    for i, im in enumerate(imgs):
        g, lap = oracle.pyramid_decompose(im, levels, oracle.binomial5(), boundary, contract=1)
        for l in range(levels - 1):
            assert np.array_equal(plan.lap(i, l).cpu().numpy(), lap[l])
    plan.close()


def test_pyramid_status_clean(gpu):
    import ctypes as C

    from hipacc_gb300 import _lib as L

    st = C.c_int(-1)
    L.call("hgb_device_status", C.byref(st))
    assert st.value == 0
