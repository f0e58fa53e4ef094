"""CPU: the oracle's FP64 hand adjoint of the bilateral filter against FP64
central differences of the oracle's FP64 forward (the bilateral body of
samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77), every
boundary mode; this pins the restatement the GPU adjoint is checked against."""
import numpy as np
import pytest


@pytest.mark.parametrize("boundary,const", [(1, 0.0), (2, 0.0), (3, 0.0), (4, 0.3)])
def test_bilateral_adjoint_oracle_vs_central_differences(oracle, boundary, const):
    rng = np.random.default_rng(boundary)
    x = rng.random((21, 17))
    g = rng.normal(0, 1, (21, 17))
    sm = oracle.spatial_mask(5, 1.2).astype(np.float64)
    sigma = 0.15
    gi, gs = oracle.bilateral_adjoint(x, g, sm, sigma, boundary, const)
    f = lambda xx, s: float(np.sum(g * oracle.bilateral(xx, sm, s, boundary, const)))
    eps = 1e-5
    for (i, j) in [(0, 0), (20, 16), (0, 8), (10, 0), (1, 15), (10, 8)]:
        xp, xm = x.copy(), x.copy()
        xp[i, j] += eps
        xm[i, j] -= eps
        fd = (f(xp, sigma) - f(xm, sigma)) / (2 * eps)
        assert abs(gi[i, j] - fd) <= 1e-6 * max(abs(fd), 1.0), (i, j, gi[i, j], fd)
    fd = (f(x, sigma + eps) - f(x, sigma - eps)) / (2 * eps)
    assert abs(gs - fd) <= 1e-6 * max(abs(fd), 1.0)
