"""Differentiable SPECT projection.

``SPECTProjectFn`` wraps the fused forward projector of a ``SPECTSystemMatrix`` in a
``torch.autograd.Function`` whose backward is the exact transpose of the forward (the
adjoint kernels: same bilinear taps, the plan's attenuation factors, PSF applied as its
own transpose).  Nothing of a forward call is kept for the backward except the system
matrix and the subset: the backward recomputes the whole operator chain from the
gradient.  A batch of objects ([B, Lx, Ly, Lz]) on one system matrix runs as one C batch
(``gb_spect_batch_forward`` / ``gb_spect_batch_backward``): one persistent forward launch
and one adjoint pass cover all B objects.  The reference has no differentiable path (its
transforms run under ``torch.no_grad``); gradients agree with torch autograd through the
reference's undecorated rotate / attenuation / PSF operations.
"""
from __future__ import annotations

import torch

import pytomography_gb300 as _p

from .batched import MAX_BATCH, BatchedOSEM, SpectBatch


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


class SPECTProjectBatchFn(torch.autograd.Function):
    """proj[b] = H_m f[b] for a batch of objects on one plan, one launch per phase."""

    @staticmethod
    def forward(ctx, objects, batch, subset_idx=None):
        ctx.batch = batch
        ctx.subset_idx = subset_idx
        sm = batch.sms[0]
        out = torch.empty((objects.shape[0], sm._n_sel(subset_idx), *sm.proj_meta.shape[1:]),
                          device=objects.device, dtype=torch.float32)
        batch.forward(list(objects.detach().contiguous()), subset_idx, out=out)
        return out

    @staticmethod
    def backward(ctx, grad_proj):
        g = grad_proj.contiguous()
        out = torch.empty((g.shape[0], *ctx.batch.sms[0].object_meta.shape), device=g.device,
                          dtype=torch.float32)
        ctx.batch.backward(list(g), ctx.subset_idx, adjoint=True, out=out)
        return out, None, None


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


def _batch_for(system_matrix, n: int):
    """The cached C batch of n entries on this system matrix, or None when the plan cannot
    be batched (no PSF, larger than 128^3, nz % 4 != 0) or n is too large."""
    if n < 2 or n > MAX_BATCH or not BatchedOSEM._batchable(system_matrix):
        return None
    cache = system_matrix.__dict__.setdefault("_autograd_batches", {})
    key = (n, system_matrix._plan.value, system_matrix._lists_epoch)
    b = cache.get(key)
    if b is None:
        cache.clear()
        b = cache[key] = SpectBatch([system_matrix] * n)
    return b


def project(object: torch.Tensor, system_matrix, subset_idx=None) -> torch.Tensor:
    """Differentiable H_m f.  A leading batch dimension projects all objects in one batched
    launch when the plan allows it (object by object otherwise)."""
    if object.dim() == 4:
        b = _batch_for(system_matrix, object.shape[0])
        if b is not None:
            return SPECTProjectBatchFn.apply(object.to(torch.float32), b, subset_idx)
        return torch.stack([SPECTProjectFn.apply(o, system_matrix, subset_idx) for o in object])
    return SPECTProjectFn.apply(object, system_matrix, subset_idx)


def poisson_nll(object: torch.Tensor, system_matrix, projections: torch.Tensor,
                additive: torch.Tensor | None = None, subset_idx=None) -> torch.Tensor:
    """sum(H f + s - g log(H f + s + delta)); its gradient is H^T (1 - g/(Hf + s + delta))."""
    pred = project(object, system_matrix, subset_idx)
    if additive is not None:
        pred = pred + additive
    return (pred - projections * torch.log(pred + _p.delta)).sum()
