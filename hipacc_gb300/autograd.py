"""Thin torch.autograd.Function over hgb_conv_bilateral_mse, used only to
check the hand-written adjoint kernels against autograd-style finite
differences.  Forward and adjoint both run in the C ABI call; backward only
scales the stored gradients by the incoming loss gradient."""
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
