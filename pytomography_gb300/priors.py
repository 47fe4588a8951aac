"""Relative-difference prior on the GPU.

Mirror of ``Prior`` (src/pytomography/priors/prior.py:7-57),
``RelativeDifferencePrior`` and ``EuclideanNeighbourWeight``
(src/pytomography/priors/nearest_neighbour.py:12-110, 156-183, 207-220).  The first-order
gradient (the BSREM hot path) is the ``gb_rdp_gradient`` CUDA kernel; inside the fused
BSREM step it is evaluated in the update epilogue.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

import pytomography_gb300 as _p

from . import _lib


class Prior:
    def __init__(self, beta: float, obj2obj_transforms=None) -> None:
        self.beta = beta
        self.obj2obj_transforms = []
        self.device = _p.device
        self.FOV_scale = None

    def set_object_meta(self, object_meta) -> None:
        self.object_meta = object_meta

    def set_beta_scale(self, factor: float) -> None:
        self.beta_scale_factor = factor

    def set_FOV_scale(self, FOV_scale: torch.Tensor) -> None:
        self.FOV_scale = FOV_scale

    def set_object(self, object: torch.Tensor) -> None:
        self.object = object.clone()


class EuclideanNeighbourWeight:
    """w_rs = dx / ||(i dx, j dy, k dz)||."""

    def set_object_meta(self, object_meta) -> None:
        self.object_meta = object_meta

    def __call__(self, coords):
        i, j, k = coords
        om = self.object_meta
        return om.dx / np.sqrt((om.dx * i) ** 2 + (om.dy * j) ** 2 + (om.dz * k) ** 2)


class RelativeDifferencePrior(Prior):
    """phi0 = (fr-fs)^2 / (fr + fs + gamma |fr-fs| + delta)."""

    def __init__(self, beta: float, weight=None, gamma: float = 1, delta: float = 1e-11) -> None:
        super().__init__(beta)
        if weight is not None and not isinstance(weight, EuclideanNeighbourWeight):
            raise NotImplementedError("only Euclidean neighbour weights are fused")
        self.weight = EuclideanNeighbourWeight()
        self.gamma = gamma
        self.delta = delta

    def set_object_meta(self, object_meta) -> None:
        self.weight.set_object_meta(object_meta)
        self.object_meta = object_meta
        self.FOV_scale = torch.ones(tuple(object_meta.shape)).to(_p.device)

    def _desc(self):
        fov = self.FOV_scale
        if fov is not None:
            fov = fov.to(torch.float32).contiguous()
            self._fov_keep = fov
        return _lib.RdpDesc(float(self.beta), float(self.gamma), float(self.delta),
                            None if fov is None else ctypes.c_void_p(fov.data_ptr()))

    def gradient(self, object: torch.Tensor, beta_scale: float = 1.0) -> torch.Tensor:
        lib = _lib.load()
        f = object.to(torch.float32).contiguous()
        _lib.require_cuda(f, "object")
        out = torch.empty_like(f)
        d = self._desc()
        dx, dy, dz = (float(v) for v in self.object_meta.dr)
        _lib.check(lib.gb_rdp_gradient(_lib.ptr(f), _lib.ptr(out), *f.shape, dx, dy, dz,
                                       ctypes.byref(d), float(beta_scale),
                                       _lib.stream_handle(f.device)))
        return out

    def _value(self) -> float:
        f = self.object
        fp = torch.nn.functional.pad(f[None, None], (1, 1, 1, 1, 1, 1), mode="replicate")[0, 0]
        nx, ny, nz = f.shape
        tot = torch.zeros((), device=f.device, dtype=torch.float64)
        for i in (-1, 0, 1):
            for j in (-1, 0, 1):
                for k in (-1, 0, 1):
                    if i == j == k == 0:
                        continue
                    fs = fp[1 + i:1 + i + nx, 1 + j:1 + j + ny, 1 + k:1 + k + nz]
                    phi = (f - fs) ** 2 / (f + fs + self.gamma * torch.abs(f - fs) + self.delta)
                    tot += (phi * float(self.weight((i, j, k))) * self.FOV_scale).sum()
        return float(self.beta * tot)

    def hessian_vector(self, x: torch.Tensor, beta_scale: float = 1.0) -> torch.Tensor:
        """Second derivative at the current object applied to ``x``
        (gb_rdp_hessian_vector)."""
        lib = _lib.load()
        f = self.object.to(torch.float32).contiguous()
        _lib.require_cuda(f, "object")
        xv = x.to(f.device, torch.float32).contiguous()
        out = torch.empty_like(f)
        d = self._desc()
        dx, dy, dz = (float(v) for v in self.object_meta.dr)
        _lib.check(lib.gb_rdp_hessian_vector(_lib.ptr(f), _lib.ptr(xv), _lib.ptr(out), *f.shape,
                                             dx, dy, dz, ctypes.byref(d), float(beta_scale),
                                             _lib.stream_handle(f.device)))
        return out

    def __call__(self, derivative_order: int = 0):
        if derivative_order == 0:
            return self._value()
        if derivative_order == 1:
            return self.gradient(self.object, self.beta_scale_factor)
        if derivative_order == 2:  # an operator, as in nearest_neighbour.py:105-108
            scale = self.beta_scale_factor
            return lambda x: self.hessian_vector(x, scale)
        raise NotImplementedError("prior derivatives of order > 2 are not defined")
