"""Thin torch.autograd.Function wrappers over the C ABI, used only to check the
hand-written adjoint kernels: ConvBilateralMSE over hgb_conv_bilateral_mse
(forward and adjoint in one call; backward scales the stored gradients by
the incoming loss gradient) and Bilateral over hgb_bilateral /
hgb_bilateral_adjoint."""
import torch

from . import api


class ConvBilateralMSE(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, t, mask, sigma, smask, boundary):
        loss, gx, gm, gs = api.conv_bilateral_mse(x, t, mask, sigma, smask, boundary)
        ctx.save_for_backward(gx, gm, gs)
        return loss.to(torch.float32)

    @staticmethod
    def backward(ctx, g):
        gx, gm, gs = ctx.saved_tensors
        g = g.to(torch.float32)
        return g * gx, None, g * gm, g * gs, None, None


class Bilateral(torch.autograd.Function):
    """y = bilateral(x; smask, sigma_r) with hgb_bilateral forward and
    hgb_bilateral_adjoint backward (gradients for x and sigma_r, a 1-element
    tensor)."""

    @staticmethod
    def forward(ctx, x, sigma, smask, boundary, const=0.0):
        s = float(sigma.item())
        ctx.save_for_backward(x)
        ctx.args = (smask, s, boundary, const)
        return api.bilateral(x, smask=smask, sigma_r=s, boundary=boundary, const=const)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        smask, s, boundary, const = ctx.args
        gi, gs = api.bilateral_adjoint(x, g.contiguous(), smask, s, boundary, const)
        return gi, gs, None, None, None
