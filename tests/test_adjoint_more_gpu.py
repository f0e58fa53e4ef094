"""GPU adjoints of the separable filter and of the MIN / MAX local operator,
against FP64 restatements of their definitions.

Separable: the forward is t = rows(in), out = cols(t), each a 1-D SUM local
operator with the boundary; the reference adjoint applies each 1-D transpose
by scattering every tap's contribution to the pixel it read (CONSTANT taps
send nothing, and read 0 in the tap gradients).

MIN / MAX: the forward starts at FLT_MAX / FLT_MIN and takes
acc = acc < v ? acc : v (MIN) or acc > v ? acc : v (MAX) per tap in row-major
order; the gradient of each output goes to the pixel read by the tap that last
replaced the running value (times its mask weight), nothing when no tap did or
when a CONSTANT tap outside won.  The restatement runs that rule in float32
exactly as the forward does, and the test checks its values against the
library's own forward first."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FLT_MIN = np.float32(1.17549435e-38)
FLT_MAX = np.float32(3.40282347e38)


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
            np.add.at(gin, (ry[Y], rx[X]), float(mask[my, mx]) * gout[Y, X])
            gm[my, mx] = np.sum(gout[Y, X] * img[ry[Y], rx[X]])
    return gin, gm


def rows64(oracle, img, taps, mode, const):
    h, w = img.shape
    k = len(taps)
    t = np.zeros((h, w))
    xs = np.arange(w)
    for j in range(k):
        rx = remap_vec(oracle, mode, xs + j - k // 2, w)
        vals = np.where((rx >= 0)[None, :], img[:, np.clip(rx, 0, w - 1)].astype(np.float64), const)
        t += float(taps[j]) * vals
    return t


def sep_adjoint64(oracle, img, gout, row, col, mode, const):
    t = rows64(oracle, img.astype(np.float64), row, mode, const)
    gt, gcol = scatter_adjoint(oracle, t, gout.astype(np.float64), np.asarray(col).reshape(-1, 1), mode)
    gin, grow = scatter_adjoint(oracle, img.astype(np.float64), gt, np.asarray(row).reshape(1, -1), mode)
    return gin, grow.ravel(), gcol.ravel()


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / max(float(np.max(np.abs(b))), 1e-30))


@pytest.mark.parametrize("k", [3, 5, 9])
@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_separable_adjoint(gpu, oracle, k, mode):
    rng = np.random.default_rng(hash((k, mode)) % 2**32)
    h, w = 37, 53
    img = rng.random((h, w)).astype(np.float32)
    gout = rng.normal(0, 1, (h, w)).astype(np.float32)
    row = rng.normal(0, 1, k).astype(np.float32)
    col = rng.normal(0, 1, k).astype(np.float32)
    gi, gr, gc = gpu.separable_adjoint(torch.from_numpy(img).cuda(), torch.from_numpy(gout).cuda(), row, col,
                                       boundary=mode, const=0.5)
    torch.cuda.synchronize()
    ref_in, ref_row, ref_col = sep_adjoint64(oracle, img, gout, row, col, mode, 0.5)
    assert rel(gi.cpu().numpy(), ref_in) <= 2e-6
    assert rel(gr.cpu().numpy(), ref_row) <= 1e-5
    assert rel(gc.cpu().numpy(), ref_col) <= 1e-5


def test_separable_adjoint_transpose_identity_and_batch(gpu, oracle):
    """<sep(x), y> = <x, sep^T(y)> with the library's own forward, on a batch
    of three images, and each image's gradients as in the single-image call."""
    rng = np.random.default_rng(5)
    taps = oracle.gaussian_taps(7, 1.5)
    x = torch.from_numpy(rng.random((3, 64, 96)).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.normal(0, 1, (3, 64, 96)).astype(np.float32)).cuda()
    for mode in (1, 2, 3):
        fx = gpu.separable(x, torch.empty_like(x), taps, taps, boundary=mode)
        gi, gr, gc = gpu.separable_adjoint(x, y, taps, taps, boundary=mode)
        torch.cuda.synchronize()
        lhs = float((fx.double() * y.double()).sum())
        rhs = float((x.double() * gi.double()).sum())
        assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), 1.0), (mode, lhs, rhs)
        ref_in, ref_row, ref_col = zip(*[sep_adjoint64(oracle, x[b].cpu().numpy(), y[b].cpu().numpy(), taps, taps,
                                                       mode, 0.0) for b in range(3)])
        assert rel(gi.cpu().numpy(), np.stack(ref_in)) <= 2e-6
        assert rel(gr.cpu().numpy(), np.sum(ref_row, axis=0)) <= 1e-5
        assert rel(gc.cpu().numpy(), np.sum(ref_col, axis=0)) <= 1e-5


def minmax64(oracle, img, gout, red_max, mode, const, mask=None, domain=None, size=None):
    h, w = img.shape
    if mask is not None:
        mh, mw = mask.shape
    elif domain is not None:
        mh, mw = domain.shape
    else:
        mh = mw = size
    acc = np.full((h, w), FLT_MIN if red_max else FLT_MAX, np.float32)
    win = np.full((h, w), -1, np.int64)
    sy = np.zeros((h, w), np.int64)
    sx = np.zeros((h, w), np.int64)
    ys, xs = np.arange(h), np.arange(w)
    for my in range(mh):
        ry = remap_vec(oracle, mode, ys + my - mh // 2, h)
        for mx in range(mw):
            if domain is not None and not domain[my, mx]:
                continue
            rx = remap_vec(oracle, mode, xs + mx - mw // 2, w)
            outside = (ry[:, None] < 0) | (rx[None, :] < 0)
            RY = np.broadcast_to(np.clip(ry, 0, h - 1)[:, None], (h, w))
            RX = np.broadcast_to(np.clip(rx, 0, w - 1)[None, :], (h, w))
            xv = np.where(outside, np.float32(const), img[RY, RX]).astype(np.float32)
            v = (np.float32(mask[my, mx]) * xv).astype(np.float32) if mask is not None else xv
            keep = acc > v if red_max else acc < v
            upd = ~keep
            acc = np.where(upd, v, acc)
            win = np.where(upd, np.where(outside, -1, my * mw + mx), win)
            sy = np.where(upd, RY, sy)
            sx = np.where(upd, RX, sx)
    gin = np.zeros((h, w))
    ok = win >= 0
    fac = np.ones(win.shape) if mask is None else mask.ravel()[np.maximum(win, 0)].astype(np.float64)
    np.add.at(gin, (sy[ok], sx[ok]), (fac * gout.astype(np.float64))[ok])
    return acc, gin


CROSS = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], np.uint8)


@pytest.mark.parametrize("red_max", [False, True])
@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("kind", ["cross", "dom5", "mask3", "ints"])
def test_minmax_adjoint(gpu, oracle, red_max, mode, kind):
    rng = np.random.default_rng(100 * int(red_max) + 10 * mode + ["cross", "dom5", "mask3", "ints"].index(kind))
    h, w = 29, 41
    img = rng.random((h, w)).astype(np.float32) - 0.25
    mask = domain = None
    if kind == "cross":
        domain = CROSS
    elif kind == "dom5":
        domain = (rng.random((5, 5)) < 0.6).astype(np.uint8)
        domain[2, 2] = 1
    elif kind == "mask3":
        mask = rng.normal(0, 1, (3, 3)).astype(np.float32)
    else:  # small integers: ties between taps, and all-zero neighbourhoods for MAX
        img = rng.integers(0, 4, (h, w)).astype(np.float32)
        domain = np.ones((3, 3), np.uint8)
    gout = rng.normal(0, 1, (h, w)).astype(np.float32)
    red = gpu.MAX if red_max else gpu.MIN
    ti = torch.from_numpy(img).cuda()
    fwd = gpu.local_op(ti, mask=mask, domain=domain, reduce=red, boundary=mode, const=0.125)
    gi = gpu.minmax_adjoint(ti, torch.from_numpy(gout).cuda(), red, mask=mask, domain=domain, boundary=mode,
                            const=0.125)
    torch.cuda.synchronize()
    acc, ref = minmax64(oracle, img, gout, red_max, mode, 0.125, mask=mask, domain=domain)
    assert np.array_equal(fwd.cpu().numpy(), acc), "the restated rule disagrees with the library's forward"
    assert rel(gi.cpu().numpy(), ref) <= 2e-6 or np.max(np.abs(ref)) == 0.0


def test_minmax_adjoint_batch(gpu, oracle):
    rng = np.random.default_rng(9)
    img = rng.random((2, 30, 50)).astype(np.float32)
    gout = rng.normal(0, 1, (2, 30, 50)).astype(np.float32)
    gi = gpu.minmax_adjoint(torch.from_numpy(img).cuda(), torch.from_numpy(gout).cuda(), gpu.MAX, domain=CROSS,
                            boundary=gpu.MIRROR)
    torch.cuda.synchronize()
    for b in range(2):
        _, ref = minmax64(oracle, img[b], gout[b], True, 3, 0.0, domain=CROSS)
        assert rel(gi[b].cpu().numpy(), ref) <= 2e-6


def test_autograd_wrappers(gpu, oracle):
    """Separable and LocalMinMax as torch.autograd.Functions: backward gives the
    adjoint entry points' gradients, which match the FP64 restatements."""
    from hipacc_gb300.autograd import LocalMinMax, Separable

    rng = np.random.default_rng(21)
    img = rng.random((40, 64)).astype(np.float32)
    wgt = rng.normal(0, 1, (40, 64)).astype(np.float32)
    x = torch.from_numpy(img).cuda().requires_grad_(True)
    w = torch.from_numpy(wgt).cuda()
    row = torch.from_numpy(rng.normal(0, 1, 5).astype(np.float32)).cuda().requires_grad_(True)
    col = torch.from_numpy(rng.normal(0, 1, 5).astype(np.float32)).cuda().requires_grad_(True)
    (Separable.apply(x, row, col, gpu.MIRROR) * w).sum().backward()
    ref_in, ref_row, ref_col = sep_adjoint64(oracle, img, wgt, row.detach().cpu().numpy(),
                                             col.detach().cpu().numpy(), 3, 0.0)
    assert rel(x.grad.cpu().numpy(), ref_in) <= 2e-6
    assert rel(row.grad.cpu().numpy(), ref_row) <= 1e-5 and rel(col.grad.cpu().numpy(), ref_col) <= 1e-5
    x.grad = None
    (LocalMinMax.apply(x, gpu.MAX, CROSS, None, gpu.REPEAT) * w).sum().backward()
    _, ref = minmax64(oracle, img, wgt, True, 2, 0.0, domain=CROSS)
    assert rel(x.grad.cpu().numpy(), ref) <= 2e-6
