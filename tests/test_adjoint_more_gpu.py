"""GPU adjoints of the separable filter and of the MIN / MAX local operator,
against the oracle's FP64 restatements of their definitions
(oracle.separable_adjoint, oracle.minmax_adjoint; tests/test_oracle_adjoint.py
pins both on the CPU: the separable one is the exact transpose of the
oracle's forward, the MIN / MAX rule reproduces the reference's forward).
The MIN / MAX test also checks the rule's values against the library's own
forward."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


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
    ref_in, ref_row, ref_col = oracle.separable_adjoint(img, gout, row, col, mode, 0.5)
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
        ref_in, ref_row, ref_col = zip(*[oracle.separable_adjoint(x[b].cpu().numpy(), y[b].cpu().numpy(), taps,
                                                                  taps, mode, 0.0) for b in range(3)])
        assert rel(gi.cpu().numpy(), np.stack(ref_in)) <= 2e-6
        assert rel(gr.cpu().numpy(), np.sum(ref_row, axis=0)) <= 1e-5
        assert rel(gc.cpu().numpy(), np.sum(ref_col, axis=0)) <= 1e-5


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
    acc, ref = oracle.minmax_adjoint(img, gout, red, mask=mask, domain=domain, boundary=mode, const=0.125)
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
        _, ref = oracle.minmax_adjoint(img[b], gout[b], gpu.MAX, domain=CROSS, boundary=3)
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
    ref_in, ref_row, ref_col = oracle.separable_adjoint(img, wgt, row.detach().cpu().numpy(),
                                                        col.detach().cpu().numpy(), 3, 0.0)
    assert rel(x.grad.cpu().numpy(), ref_in) <= 2e-6
    assert rel(row.grad.cpu().numpy(), ref_row) <= 1e-5 and rel(col.grad.cpu().numpy(), ref_col) <= 1e-5
    x.grad = None
    (LocalMinMax.apply(x, gpu.MAX, CROSS, None, gpu.REPEAT) * w).sum().backward()
    _, ref = oracle.minmax_adjoint(img, wgt, gpu.MAX, domain=CROSS, boundary=2)
    assert rel(x.grad.cpu().numpy(), ref) <= 2e-6
