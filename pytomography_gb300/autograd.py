"""Differentiable SPECT projection.

``SPECTProjectFn`` wraps the fused forward projector of a ``SPECTSystemMatrix`` in a
``torch.autograd.Function`` whose backward is the exact transpose of the forward (the
adjoint kernels: same bilinear taps, attenuation factors recomputed from the plan's
table, PSF applied as its own transpose).  The reference has no differentiable path
(its transforms run under ``torch.no_grad``); gradients agree with torch autograd
through the reference's undecorated rotate / attenuation / PSF operations.
"""
from __future__ import annotations

import torch

import pytomography_gb300 as _p


class SPECTProjectFn(torch.autograd.Function):
    """proj = H_m f, d/df = H_m^T (exact adjoint)."""

    @staticmethod
    def forward(ctx, object, system_matrix, subset_idx=None):
        ctx.system_matrix = system_matrix
        ctx.subset_idx = subset_idx
        return system_matrix.forward(object.detach(), subset_idx)

    @staticmethod
    def backward(ctx, grad_proj):
        g = ctx.system_matrix.backward_adjoint(grad_proj.contiguous(), ctx.subset_idx)
        return g, None, None


class SPECTBackprojectFn(torch.autograd.Function):
    """obj = H_m^T g (exact adjoint), d/dg = H_m."""

    @staticmethod
    def forward(ctx, proj, system_matrix, subset_idx=None):
        ctx.system_matrix = system_matrix
        ctx.subset_idx = subset_idx
        return system_matrix.backward_adjoint(proj.detach().contiguous(), subset_idx)

    @staticmethod
    def backward(ctx, grad_obj):
        return ctx.system_matrix.forward(grad_obj.contiguous(), ctx.subset_idx), None, None


def project(object: torch.Tensor, system_matrix, subset_idx=None) -> torch.Tensor:
    """Differentiable H_m f.  A leading batch dimension is projected object by object."""
    if object.dim() == 4:
        return torch.stack([SPECTProjectFn.apply(o, system_matrix, subset_idx) for o in object])
    return SPECTProjectFn.apply(object, system_matrix, subset_idx)


def poisson_nll(object: torch.Tensor, system_matrix, projections: torch.Tensor,
                additive: torch.Tensor | None = None, subset_idx=None) -> torch.Tensor:
    """sum(H f + s - g log(H f + s + delta)); its gradient is H^T (1 - g/(Hf + s + delta))."""
    pred = project(object, system_matrix, subset_idx)
    if additive is not None:
        pred = pred + additive
    return (pred - projections * torch.log(pred + _p.delta)).sum()
