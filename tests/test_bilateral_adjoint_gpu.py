"""GPU: hgb_bilateral_adjoint, the adjoint of the bilateral filter
(samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77), against
the FP64 oracle's hand adjoint (itself pinned to FP64 central differences in
test_oracle_adjoint.py) and against FP64 central differences (eps = 1e-4) of
the FP64 forward on 64x64 crops.  The kernels evaluate the range weights with
the FP32 exp2 instruction and accumulate in FP32, so gradients agree with FP64
to ADJ_TOL relative (L2 norm over the image) and dL/dsigma_r to ADJ_TOL
relative, with an absolute floor of SIGMA_ABS where its terms cancel to a
small total (FP32 sums of terms of both signs)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ADJ_TOL = 2e-3
SIGMA_ABS = 1e-4
FD_TOL = 5e-3


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


def _gpu(api, x, g, sm, sigma, boundary, const):
    gi, gs = api.bilateral_adjoint(torch.from_numpy(x).cuda(), torch.from_numpy(g).cuda(), sm, sigma, boundary, const)
    torch.cuda.synchronize()
    return gi.cpu().numpy(), float(gs.item())


@pytest.mark.parametrize("boundary,const", [(0, 0.0), (1, 0.0), (2, 0.0), (3, 0.0), (4, 0.5)])
@pytest.mark.parametrize("size,hw", [(5, (64, 64)), (9, (97, 150)), (13, (40, 33))])
def test_bilateral_adjoint_vs_fp64_oracle(gpu, oracle, boundary, const, size, hw):
    rng = np.random.default_rng(size * 10 + boundary)
    B = 2
    h, w = hw
    x = rng.random((B, h, w), dtype=np.float32)
    g = rng.normal(0, 1, (B, h, w)).astype(np.float32)
    sm = oracle.spatial_mask(size, size / 4.0)
    sigma = 0.15
    gi, gs = _gpu(gpu, x, g, sm, sigma, boundary, const)
    ref_gi, ref_gs = [], 0.0
    for b in range(B):
        a, s = oracle.bilateral_adjoint(x[b], g[b], sm.astype(np.float64), sigma, boundary, const)
        ref_gi.append(a)
        ref_gs += s
    assert rel(gi, np.stack(ref_gi)) <= ADJ_TOL, rel(gi, np.stack(ref_gi))
    assert abs(gs - ref_gs) <= max(ADJ_TOL * abs(ref_gs), SIGMA_ABS), (gs, ref_gs)


@pytest.mark.parametrize("boundary,const", [(1, 0.0), (2, 0.0), (3, 0.0), (4, 0.5)])
@pytest.mark.parametrize("size", [3, 7, 11])
def test_bilateral_adjoint_many_tiles(gpu, oracle, boundary, const, size):
    """Symmetric masks on images of several 64 x 16 tiles with ragged edges
    (the packed form: tiles, then the edge band by pre-images): every pixel
    of dL/din against the FP64 oracle, and dL/dsigma_r."""
    rng = np.random.default_rng(size * 100 + boundary)
    B, h, w = 2, 53, 203
    x = rng.random((B, h, w), dtype=np.float32)
    g = rng.normal(0, 1, (B, h, w)).astype(np.float32)
    sm = oracle.spatial_mask(size, size / 4.0)
    sigma = 0.2
    gi, gs = _gpu(gpu, x, g, sm, sigma, boundary, const)
    ref_gs = 0.0
    for b in range(B):
        a, sg = oracle.bilateral_adjoint(x[b], g[b], sm.astype(np.float64), sigma, boundary, const)
        ref_gs += sg
        err = np.abs(gi[b] - a)
        assert np.max(err) <= 2e-3 * np.max(np.abs(a)), (b, np.unravel_index(np.argmax(err), err.shape))
    assert abs(gs - ref_gs) <= max(ADJ_TOL * abs(ref_gs), SIGMA_ABS), (gs, ref_gs)


@pytest.mark.parametrize("boundary", [1, 3])
def test_bilateral_adjoint_vs_central_differences(gpu, oracle, boundary):
    """L = sum(g * bilateral(x)) in FP64; central differences with eps = 1e-4
    at corners, edges and interior points of a 64x64 crop, and in sigma_r."""
    rng = np.random.default_rng(70 + boundary)
    x = rng.random((64, 64), dtype=np.float32)
    g = rng.normal(0, 1, (64, 64)).astype(np.float32)
    sm = oracle.spatial_mask(9, 2.0)
    sigma = 0.15
    gi, gs = _gpu(gpu, x, g, sm, sigma, boundary, 0.0)
    x64, g64, s64 = x.astype(np.float64), g.astype(np.float64), sm.astype(np.float64)
    f = lambda xx, s: float(np.sum(g64 * oracle.bilateral(xx, s64, s, boundary)))
    eps = 1e-4
    for (i, j) in [(0, 0), (0, 63), (63, 0), (63, 63), (1, 2), (31, 32), (5, 60), (60, 4)]:
        xp, xm = x64.copy(), x64.copy()
        xp[i, j] += eps
        xm[i, j] -= eps
        fd = (f(xp, sigma) - f(xm, sigma)) / (2 * eps)
        assert abs(gi[i, j] - fd) <= FD_TOL * max(abs(fd), 1e-3), (i, j, gi[i, j], fd)
    fd = (f(x64, sigma + eps) - f(x64, sigma - eps)) / (2 * eps)
    assert abs(gs - fd) <= FD_TOL * abs(fd), (gs, fd)


def test_bilateral_adjoint_asymmetric_mask(gpu, oracle):
    """A spatial mask without point symmetry (and a zero cell) takes the
    general gather everywhere."""
    rng = np.random.default_rng(5)
    x = rng.random((1, 48, 70), dtype=np.float32)
    g = rng.normal(0, 1, (1, 48, 70)).astype(np.float32)
    sm = rng.random((7, 7)).astype(np.float32)
    sm[0, 3] = 0.0
    for boundary in (1, 2, 3):
        gi, gs = _gpu(gpu, x, g, sm, 0.2, boundary, 0.0)
        a, s = oracle.bilateral_adjoint(x[0], g[0], sm.astype(np.float64), 0.2, boundary, 0.0)
        assert rel(gi[0], a) <= ADJ_TOL, boundary
        assert abs(gs - s) <= max(ADJ_TOL * abs(s), SIGMA_ABS), (boundary, gs, s)


def test_bilateral_adjoint_partial_requests_and_errors(gpu, oracle):
    from hipacc_gb300 import _lib as L

    rng = np.random.default_rng(6)
    x = torch.from_numpy(rng.random((32, 40), dtype=np.float32)).cuda()
    g = torch.from_numpy(rng.normal(0, 1, (32, 40)).astype(np.float32)).cuda()
    sm = oracle.spatial_mask(5, 1.0)
    gi_a, gs_a = gpu.bilateral_adjoint(x, g, sm, 0.1, 3)
    gi_b, _ = gpu.bilateral_adjoint(x, g, sm, 0.1, 3, want_grad_sigma=False)
    _, gs_c = gpu.bilateral_adjoint(x, g, sm, 0.1, 3, want_grad_in=False)
    torch.cuda.synchronize()
    assert torch.equal(gi_a, gi_b) and float(gs_a.item()) == float(gs_c.item())  # deterministic
    with pytest.raises(L.HgbError):
        gpu.bilateral_adjoint(x, g, sm, 0.1, 3, want_grad_in=False, want_grad_sigma=False)
    with pytest.raises(L.HgbError):
        gpu.bilateral_adjoint(x, g, np.ones((4, 4), np.float32), 0.1, 3)
    with pytest.raises(L.HgbError):
        gpu.bilateral_adjoint(x, g, sm, -0.1, 3)


def test_bilateral_autograd_wrapper(gpu, oracle):
    from hipacc_gb300.autograd import Bilateral

    rng = np.random.default_rng(8)
    x = torch.from_numpy(rng.random((40, 56), dtype=np.float32)).cuda().requires_grad_(True)
    s = torch.tensor([0.12], device="cuda", requires_grad=True)
    w = torch.from_numpy(rng.normal(0, 1, (40, 56)).astype(np.float32)).cuda()
    sm = oracle.spatial_mask(7, 1.5)
    y = Bilateral.apply(x, s, sm, 1)
    (y * w).sum().backward()
    a, gs = oracle.bilateral_adjoint(x.detach().cpu().numpy(), w.cpu().numpy(), sm.astype(np.float64), 0.12, 1)
    assert rel(x.grad.cpu().numpy(), a) <= ADJ_TOL
    assert abs(s.grad.item() - gs) <= ADJ_TOL * abs(gs)
