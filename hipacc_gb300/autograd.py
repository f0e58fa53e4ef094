"""Thin torch.autograd.Function wrappers over the C ABI, used only to check the
hand-written adjoint kernels: ConvBilateralMSE over hgb_conv_bilateral_mse
(forward and adjoint in one call; backward scales the stored gradients by
the incoming loss gradient), Bilateral over hgb_bilateral /
hgb_bilateral_adjoint, Separable over hgb_separable / hgb_separable_adjoint
and LocalMinMax over hgb_local_op (MIN / MAX) / hgb_local_op_minmax_adjoint."""
import numpy as np
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


class Separable(torch.autograd.Function):
    """y = separable(x; row, col) (FP32) with gradients for x and for both tap
    vectors (1-D float32 tensors on any device; the forward reads them on the
    host)."""

    @staticmethod
    def forward(ctx, x, row, col, boundary, const=0.0):
        r = row.detach().float().cpu().numpy()
        c = col.detach().float().cpu().numpy()
        ctx.save_for_backward(x)
        ctx.args = (r, c, boundary, const, row.device, col.device)
        return api.separable(x, torch.empty_like(x), r, c, boundary=boundary, const=const)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        r, c, boundary, const, rdev, cdev = ctx.args
        gi, gr, gc = api.separable_adjoint(x, g.contiguous(), r, c, boundary=boundary, const=const)
        return gi, gr.to(rdev), gc.to(cdev), None, None


class LocalMinMax(torch.autograd.Function):
    """y = MIN / MAX local operator of x over a Domain (or with a mask, as
    convolve does); the gradient goes to each output's winning pixel."""

    @staticmethod
    def forward(ctx, x, reduce, domain=None, mask=None, boundary=api.CLAMP, const=0.0):
        d = None if domain is None else np.ascontiguousarray(domain, np.uint8)
        m = None if mask is None else np.ascontiguousarray(mask, np.float32)
        ctx.save_for_backward(x)
        ctx.args = (reduce, d, m, boundary, const)
        return api.local_op(x, mask=m, domain=d, reduce=reduce, boundary=boundary, const=const)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        reduce, d, m, boundary, const = ctx.args
        gi = api.minmax_adjoint(x, g.contiguous(), reduce, mask=m, domain=d, boundary=boundary, const=const)
        return gi, None, None, None, None, None
