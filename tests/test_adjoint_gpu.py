"""GPU forward + adjoint of conv7x7 -> bilateral9x9 -> MSE against the FP64
oracle (hand adjoint, itself pinned to FP64 central differences) and FP64
central differences (eps = 1e-4) on 64x64 crops.  Tolerances: the kernels
evaluate the range weights with the FP32 exp2 instruction and accumulate in
FP32, so gradients agree with FP64 to ADJ_TOL relative (L2 norm) and the
loss to LOSS_TOL."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ADJ_TOL = 2e-3
LOSS_TOL = 1e-4


def _setup(oracle, B, H, W, boundary, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((B, H, W), dtype=np.float32)
    g15 = oracle.gaussian_mask(7, 1.5)
    t = np.stack([oracle.local_op(x[i], mask=g15, boundary=boundary) for i in range(B)]).astype(np.float32)
    mask = rng.normal(0, 0.02, (7, 7)).astype(np.float32)
    mask[3, 3] += 0.8  # a trained-like mask so that y1 is not near zero
    sm = oracle.spatial_mask(9, 2.0)
    return x, t, mask, sm


def _gpu(api, x, t, mask, sigma, sm, boundary, mode):
    loss, gx, gm, gs = api.conv_bilateral_mse(torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda(),
                                              torch.from_numpy(mask).cuda(),
                                              torch.tensor([sigma], dtype=torch.float32, device="cuda"), sm, boundary,
                                              mode)
    torch.cuda.synchronize()
    return float(loss.item()), gx.cpu().numpy(), gm.cpu().numpy(), float(gs.item())


def _oracle_batch(oracle, x, t, mask, sm, sigma, boundary):
    """The batch loss is the mean over every pixel of every image."""
    B = x.shape[0]
    L, dx, dm, ds = 0.0, [], np.zeros((7, 7)), 0.0
    for i in range(B):
        l, a, b, c = oracle.c5_grad(x[i], t[i], mask.astype(np.float64), sm.astype(np.float64), sigma, boundary)
        L += l / B
        dx.append(a / B)
        dm += b / B
        ds += c / B
    return L, np.stack(dx), dm, ds


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


@pytest.mark.parametrize("boundary", [1, 3, 4])
@pytest.mark.parametrize("mode", [0, 1])
def test_adjoint_vs_fp64_oracle(gpu, oracle, boundary, mode):
    x, t, mask, sm = _setup(oracle, 2, 64, 64, boundary, 10 + boundary)
    sigma = 0.15
    L, dx, dm, ds = _gpu(gpu, x, t, mask, sigma, sm, boundary, mode)
    L0, dx0, dm0, ds0 = _oracle_batch(oracle, x, t, mask, sm, sigma, boundary)
    assert abs(L - L0) <= LOSS_TOL * abs(L0)
    assert rel(dx, dx0) <= ADJ_TOL, rel(dx, dx0)
    assert rel(dm, dm0) <= ADJ_TOL, rel(dm, dm0)
    assert abs(ds - ds0) <= ADJ_TOL * abs(ds0), (ds, ds0)


@pytest.mark.parametrize("hw", [(8, 8), (9, 13), (21, 67), (70, 131), (37, 2 * 64 + 6)])
@pytest.mark.parametrize("boundary", [1, 3, 4])
def test_adjoint_ragged_shapes(gpu, oracle, hw, boundary):
    """Images from the 8 x 8 minimum up to several tiles with ragged edges: the
    fused form splits the pixels into tiles and the edge bands (radius 4 for
    the bilateral, 3 for the convolution), the unfused form does not; both
    against the FP64 oracle."""
    H, W = hw
    x, t, mask, sm = _setup(oracle, 2, H, W, boundary, 70 + H + W + boundary)
    L0, dx0, dm0, ds0 = _oracle_batch(oracle, x, t, mask, sm, 0.15, boundary)
    for mode in (0, 1):
        L, dx, dm, ds = _gpu(gpu, x, t, mask, 0.15, sm, boundary, mode)
        assert abs(L - L0) <= LOSS_TOL * abs(L0), (mode, L, L0)
        assert rel(dx, dx0) <= ADJ_TOL, (mode, rel(dx, dx0))
        assert rel(dm, dm0) <= ADJ_TOL, (mode, rel(dm, dm0))
        assert abs(ds - ds0) <= ADJ_TOL * abs(ds0), (mode, ds, ds0)
        # no pixel off: the band pixels are a small share of the larger images
        err = np.abs(dx - dx0)
        assert np.max(err) <= 1e-4 * np.max(np.abs(dx0)), (mode, np.unravel_index(np.argmax(err), err.shape))


@pytest.mark.parametrize("boundary", [1, 3, 4])
def test_adjoint_padded_rows_equal_dense(gpu, oracle, boundary):
    """Rows padded to a pitch that is not a multiple of 16 bytes rule out the
    TMA staging: the plain-load staging must give bit-identical results."""
    x, t, mask, sm = _setup(oracle, 2, 70, 150, boundary, 90 + boundary)
    xd = torch.from_numpy(x).cuda()
    xp = torch.zeros((2, 70, 151), dtype=torch.float32, device="cuda")
    xp[:, :, :150] = xd
    args = (torch.from_numpy(t).cuda(), torch.from_numpy(mask).cuda(),
            torch.tensor([0.15], dtype=torch.float32, device="cuda"), sm, boundary, 0)
    a = gpu.conv_bilateral_mse(xd, *args)
    b = gpu.conv_bilateral_mse(xp[:, :, :150], *args)
    torch.cuda.synchronize()
    for u, v in zip(a, b):
        assert torch.equal(u, v)


@pytest.mark.parametrize("boundary", [1, 3])
def test_adjoint_vs_central_differences(gpu, oracle, boundary):
    """FP64 central differences (eps = 1e-4) of the FP64 forward on a 64x64 crop."""
    x, t, mask, sm = _setup(oracle, 1, 64, 64, boundary, 20 + boundary)
    sigma = 0.15
    _, dx, dm, ds = _gpu(gpu, x, t, mask, sigma, sm, boundary, 0)
    eps = 1e-4
    x64, t64, m64, s64 = x[0].astype(np.float64), t[0].astype(np.float64), mask.astype(np.float64), sm.astype(np.float64)
    f = lambda xx, mm, ss: oracle.c5_loss(xx, t64, mm, s64, ss, boundary)
    for (i, j) in [(0, 0), (0, 63), (63, 5), (31, 32), (2, 61)]:
        xp, xm = x64.copy(), x64.copy()
        xp[i, j] += eps
        xm[i, j] -= eps
        fd = (f(xp, m64, sigma) - f(xm, m64, sigma)) / (2 * eps)
        assert abs(dx[0, i, j] - fd) <= 5e-3 * max(abs(fd), 1e-6) + 1e-9, (i, j, dx[0, i, j], fd)
    for (i, j) in [(0, 0), (3, 3), (6, 2)]:
        mp, mm = m64.copy(), m64.copy()
        mp[i, j] += eps
        mm[i, j] -= eps
        fd = (f(x64, mp, sigma) - f(x64, mm, sigma)) / (2 * eps)
        assert abs(dm[i, j] - fd) <= 5e-3 * abs(fd), (i, j, dm[i, j], fd)
    fd = (f(x64, m64, sigma + eps) - f(x64, m64, sigma - eps)) / (2 * eps)
    assert abs(ds - fd) <= 5e-3 * abs(fd), (ds, fd)


def test_fused_equals_unfused(gpu, oracle):
    x, t, mask, sm = _setup(oracle, 3, 96, 160, 3, 30)
    a = _gpu(gpu, x, t, mask, 0.15, sm, 3, 0)
    b = _gpu(gpu, x, t, mask, 0.15, sm, 3, 1)
    assert abs(a[0] - b[0]) <= 1e-6 * abs(b[0])
    assert rel(a[1], b[1]) <= 1e-5 and rel(a[2], b[2]) <= 1e-5 and abs(a[3] - b[3]) <= 1e-5 * abs(b[3])


def test_autograd_wrapper(gpu, oracle):
    from hipacc_gb300.autograd import ConvBilateralMSE

    x, t, mask, sm = _setup(oracle, 1, 48, 40, 1, 40)
    xt = torch.from_numpy(x).cuda().requires_grad_(True)
    mt = torch.from_numpy(mask).cuda().requires_grad_(True)
    st = torch.tensor([0.15], device="cuda", requires_grad=True)
    loss = ConvBilateralMSE.apply(xt, torch.from_numpy(t).cuda(), mt, st, sm, 1)
    (2.0 * loss).backward()
    _, dx, dm, ds = _gpu(gpu, x, t, mask, 0.15, sm, 1, 0)
    assert np.allclose(xt.grad.cpu().numpy(), 2 * dx) and np.allclose(mt.grad.cpu().numpy(), 2 * dm)
    assert abs(st.grad.item() - 2 * ds) <= 1e-6 * abs(ds)


def test_adjoint_2048(gpu, oracle):
    """One 2048x2048 image of the differentiation workload against FP64."""
    x, t, mask, sm = _setup(oracle, 1, 2048, 2048, 3, 50)
    L, dx, dm, ds = _gpu(gpu, x, t, mask, 0.15, sm, 3, 0)
    L0, dx0, dm0, ds0 = _oracle_batch(oracle, x, t, mask, sm, 0.15, 3)
    assert abs(L - L0) <= LOSS_TOL * abs(L0)
    assert rel(dx, dx0) <= ADJ_TOL and rel(dm, dm0) <= ADJ_TOL and abs(ds - ds0) <= ADJ_TOL * abs(ds0)


@pytest.mark.parametrize("boundary", [1, 3])
def test_adjoint_full_batch_16x2048(gpu, oracle, boundary):
    """The differentiation workload as it is benchmarked: a batch of 16
    2048x2048 images in the fused mode.  The batch loss is the mean over every
    pixel of every image, so image b's input gradient is its single-image
    gradient divided by 16: images 0 and 15 of the batch are checked against
    the FP64 oracle that way.  The batch's loss, mask and sigma gradients must
    be the mean of the 16 single-image results (each a separate launch), and
    the single-image results of images 0 and 15 match the FP64 oracle."""
    B, H, W = 16, 2048, 2048
    rng = np.random.default_rng(60 + boundary)
    x = torch.rand((B, H, W), device="cuda", generator=torch.Generator("cuda").manual_seed(61 + boundary))
    t = torch.empty_like(x)
    gpu.local_op(x, t, mask=oracle.gaussian_mask(7, 1.5), boundary=boundary)
    mask = rng.normal(0, 0.02, (7, 7)).astype(np.float32)
    mask[3, 3] += 0.8
    sm = oracle.spatial_mask(9, 2.0)
    sigma = 0.15
    md = torch.from_numpy(mask).cuda()
    sd = torch.tensor([sigma], dtype=torch.float32, device="cuda")
    loss, gx, gm, gs = gpu.conv_bilateral_mse(x, t, md, sd, sm, boundary, 0)
    torch.cuda.synchronize()
    Lb, dmb, dsb = float(loss.item()), gm.cpu().numpy().astype(np.float64), float(gs.item())
    # the 16 single-image launches
    singles = []
    for b in range(B):
        l1, g1, m1, s1 = gpu.conv_bilateral_mse(x[b:b + 1], t[b:b + 1], md, sd, sm, boundary, 0)
        singles.append((float(l1.item()), g1, m1.cpu().numpy().astype(np.float64), float(s1.item())))
    torch.cuda.synchronize()
    assert abs(Lb - np.mean([s[0] for s in singles])) <= 1e-6 * abs(Lb)
    assert rel(dmb, np.mean([s[2] for s in singles], axis=0)) <= 1e-5
    assert abs(dsb - np.mean([s[3] for s in singles])) <= 1e-5 * abs(dsb)
    for b in (0, B - 1):
        # the batch's gradient of image b is its single-image gradient / 16
        assert rel(gx[b].cpu().numpy(), singles[b][1][0].cpu().numpy() / B) <= 1e-6
        xb, tb = x[b].cpu().numpy(), t[b].cpu().numpy()
        l0, dx0, dm0, ds0 = oracle.c5_grad(xb, tb, mask.astype(np.float64), sm.astype(np.float64), sigma, boundary)
        assert abs(singles[b][0] - l0) <= LOSS_TOL * abs(l0), (b, singles[b][0], l0)
        assert rel(gx[b].cpu().numpy(), dx0 / B) <= ADJ_TOL, (b, rel(gx[b].cpu().numpy(), dx0 / B))
        assert rel(singles[b][2], dm0) <= ADJ_TOL, (b, rel(singles[b][2], dm0))
        assert abs(singles[b][3] - ds0) <= ADJ_TOL * abs(ds0), (b, singles[b][3], ds0)
