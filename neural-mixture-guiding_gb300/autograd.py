"""torch.autograd bindings over the C ABI, for gradient checks.

GuidingNetworkFn: raw = network(x; params) with the hand-written FP32
  forward/backward kernels (nmg_infer_raw / nmg_network_vjp on the plain
  path): backward returns dL/dparams.
MixtureKLFn: the summed KL loss of the mixture on raw outputs with its
  hand-derived adjoint (nmg_mixture_loss_grad, train.cu:69-124): backward
  returns dL/draw.
kl_loss_torch: the same loss written with torch operations (activations,
  vMF pdf, mixture, KL) so that autograd provides an independent gradient of
  the hand-derived adjoint.

These exist to check gradients; the training step itself never goes through
torch.
"""
import math

import torch

from . import GuidingField, mixture_loss_grad


class GuidingNetworkFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, params, field):
        field.set_params(params.detach().contiguous())
        raw = field.infer_raw(x.contiguous(), which=0)
        ctx.field = field
        ctx.save_for_backward(x)
        return raw

    @staticmethod
    def backward(ctx, grad_raw):
        (x,) = ctx.saved_tensors
        _, dparams = ctx.field.vjp(x.contiguous(), grad_raw.contiguous().float())
        return None, dparams, None


class MixtureKLFn(torch.autograd.Function):
    """Sum over samples of the per-sample KL loss (train.cu:93)."""

    @staticmethod
    def forward(ctx, raw, records, n_lobes, kappa_poly):
        n = raw.shape[0]
        # loss_scale = n makes the kernel's gradient the derivative of the summed loss
        g, _, tot = mixture_loss_grad(raw.contiguous(), records.contiguous(), n_lobes, loss_scale=float(n),
                                      kappa_poly=kappa_poly)
        ctx.save_for_backward(g)
        return tot.to(raw.dtype).reshape(())

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return g * grad_out, None, None, None


def kl_loss_torch(raw, records, n_lobes):
    """Summed KL loss of the mixture written in torch (autograd-able): the
    activations of train.h:391-415, the vMF pdf of vmf.h:22-27, the mixture
    of distribution.h:113-119 and the loss -L/p log(q + eps) of train.cu:93."""
    K = n_lobes
    r = raw[:, :4 * K].reshape(-1, K, 4)
    lam = torch.exp(torch.clamp(r[..., 0], -10, 15))
    kap = torch.exp(torch.clamp(r[..., 1], -10, 15))
    th = math.pi * torch.sigmoid(r[..., 2])
    ph = 2 * math.pi * torch.sigmoid(r[..., 3])
    mu = torch.stack([torch.sin(th) * torch.cos(ph), torch.sin(th) * torch.sin(ph), torch.cos(th)], -1)
    w = lam / lam.sum(dim=1, keepdim=True)
    t, p = records[:, 0], records[:, 1]
    wi = torch.stack([torch.sin(t) * torch.cos(p), torch.sin(t) * torch.sin(p), torch.cos(t)], -1)
    c = (mu * wi[:, None, :]).sum(-1)
    vmf = kap * torch.exp(kap * torch.clamp(c - 1, max=0.0)) / (2 * math.pi * -torch.expm1(-2 * kap))
    q = (w * vmf).sum(1) + 1e-5
    Li = records[:, 2:5].mean(1)
    wp = records[:, 5] + 1e-5
    return (-Li / wp * torch.log(q)).sum()


__all__ = ["GuidingNetworkFn", "MixtureKLFn", "kl_loss_torch", "GuidingField"]
