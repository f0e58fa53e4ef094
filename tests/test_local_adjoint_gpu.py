"""GPU adjoint of the SUM local operator against an FP64 scatter restatement:
every tap o of every output j sends m_o * grad_out(j) to r(j + o) (CONSTANT
taps send nothing), and grad_m(o) = sum_j grad_out(j) in(r(j + o))."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def remap_vec(oracle, mode, idx, n):
    return np.array([oracle.remap(mode, int(i), 0, n) for i in idx], np.int64)


def scatter_adjoint(oracle, img, gout, mask, mode):
    h, w = gout.shape
    mh, mw = mask.shape
    gin = np.zeros((h, w))
    gm = np.zeros((mh, mw))
    ys, xs = np.arange(h), np.arange(w)
    for my in range(mh):
        ry = remap_vec(oracle, mode, ys + my - mh // 2, h)
        for mx in range(mw):
            rx = remap_vec(oracle, mode, xs + mx - mw // 2, w)
            oky, okx = ry >= 0, rx >= 0
            Y, X = np.meshgrid(np.where(oky)[0], np.where(okx)[0], indexing="ij")
            np.add.at(gin, (ry[Y], rx[X]), mask[my, mx] * gout[Y, X])
            gm[my, mx] = np.sum(gout[Y, X] * img[ry[Y], rx[X]])
    return gin, gm


@pytest.mark.parametrize("shape", [(3, 3), (5, 5), (7, 7), (4, 6), (1, 9)])
@pytest.mark.parametrize("mode", [1, 2, 3, 4])
def test_local_adjoint(gpu, oracle, shape, mode):
    rng = np.random.default_rng(hash((shape, mode)) % 2**32)
    h, w = 37, 53
    img = rng.random((h, w)).astype(np.float32)
    gout = rng.normal(0, 1, (h, w)).astype(np.float32)
    mask = rng.normal(0, 1, shape).astype(np.float32)
    gi, gm = gpu.local_op_adjoint(torch.from_numpy(gout).cuda(), mask, mode, inp=torch.from_numpy(img).cuda())
    torch.cuda.synchronize()
    rgi, rgm = scatter_adjoint(oracle, img.astype(np.float64), gout.astype(np.float64), mask.astype(np.float64), mode)
    assert np.max(np.abs(gi.cpu().numpy() - rgi)) <= 1e-4 * max(1.0, np.max(np.abs(rgi)))
    assert np.max(np.abs(gm.cpu().numpy() - rgm)) <= 1e-4 * max(1.0, np.max(np.abs(rgm)))


def test_local_adjoint_is_transpose(gpu, oracle):
    """<conv(x), g> == <x, conv^T(g)> for every boundary with a device mask."""
    rng = np.random.default_rng(3)
    x = rng.random((2, 40, 50)).astype(np.float32)
    g = rng.normal(0, 1, (2, 40, 50)).astype(np.float32)
    m = rng.normal(0, 1, (5, 5)).astype(np.float32)
    for mode in (1, 2, 3, 4):
        xt, gt = torch.from_numpy(x).cuda(), torch.from_numpy(g).cuda()
        y = gpu.local_op(xt, mask=m, boundary=mode, const=0.0)
        gi, _ = gpu.local_op_adjoint(gt, torch.from_numpy(m).cuda(), mode, want_grad_mask=False)
        lhs = float((y.double() * gt.double()).sum())
        rhs = float((xt.double() * gi.double()).sum())
        assert abs(lhs - rhs) <= 1e-4 * abs(lhs), (mode, lhs, rhs)


@pytest.mark.parametrize("k", [3, 5, 7])
@pytest.mark.parametrize("mode", [1, 2, 3, 4])
def test_local_adjoint_mask_gradient_batch(gpu, oracle, k, mode):
    """The mask gradient of a batch over many tiles (ragged edges): the sum over
    every image of the batch, deterministic from run to run."""
    rng = np.random.default_rng(hash(("b", k, mode)) % 2**32)
    B, h, w = 2, 130, 211
    img = rng.random((B, h, w)).astype(np.float32)
    gout = rng.normal(0, 1, (B, h, w)).astype(np.float32)
    mask = rng.normal(0, 1, (k, k)).astype(np.float32)
    gi, gm = gpu.local_op_adjoint(torch.from_numpy(gout).cuda(), mask, mode, inp=torch.from_numpy(img).cuda())
    _, gm2 = gpu.local_op_adjoint(torch.from_numpy(gout).cuda(), mask, mode, inp=torch.from_numpy(img).cuda())
    torch.cuda.synchronize()
    rgm = np.zeros((k, k))
    for b in range(B):
        rgi, g1 = scatter_adjoint(oracle, img[b].astype(np.float64), gout[b].astype(np.float64),
                                  mask.astype(np.float64), mode)
        rgm += g1
        assert np.max(np.abs(gi[b].cpu().numpy() - rgi)) <= 1e-4 * max(1.0, np.max(np.abs(rgi)))
    assert np.max(np.abs(gm.cpu().numpy() - rgm)) <= 1e-4 * max(1.0, np.max(np.abs(rgm)))
    assert torch.equal(gm, gm2)


@pytest.mark.parametrize("k", [3, 5, 7])
@pytest.mark.parametrize("mode", [1, 2, 3, 4])
@pytest.mark.parametrize("bhw", [(2, 70, 132), (1, 37, 64), (1, 8, 8), (3, 19, 200)])
def test_local_adjoint_fused_tiles(gpu, oracle, k, mode, bhw):
    """Rows whose pitch is a multiple of 16 bytes take the fused kernel (both
    gradients from one TMA-staged tile walk, edge bands by pre-images): every
    pixel of grad_in and the batch's mask gradient against the FP64 scatter,
    and the mask gradient the same from run to run."""
    B, h, w = bhw
    rng = np.random.default_rng(hash(("f", k, mode, bhw)) % 2**32)
    img = rng.random((B, h, w)).astype(np.float32)
    gout = rng.normal(0, 1, (B, h, w)).astype(np.float32)
    mask = rng.normal(0, 1, (k, k)).astype(np.float32)
    gi, gm = gpu.local_op_adjoint(torch.from_numpy(gout).cuda(), mask, mode, inp=torch.from_numpy(img).cuda())
    _, gm2 = gpu.local_op_adjoint(torch.from_numpy(gout).cuda(), torch.from_numpy(mask).cuda(), mode,
                                  inp=torch.from_numpy(img).cuda())
    torch.cuda.synchronize()
    rgm = np.zeros((k, k))
    for b in range(B):
        rgi, g1 = scatter_adjoint(oracle, img[b].astype(np.float64), gout[b].astype(np.float64),
                                  mask.astype(np.float64), mode)
        rgm += g1
        assert np.max(np.abs(gi[b].cpu().numpy() - rgi)) <= 1e-4 * max(1.0, np.max(np.abs(rgi))), b
    assert np.max(np.abs(gm.cpu().numpy() - rgm)) <= 1e-4 * max(1.0, np.max(np.abs(rgm)))
    assert torch.equal(gm, gm2)
