"""SystemMatrix base class (src/pytomography/projectors/system_matrix.py:10-115)."""
from __future__ import annotations

import abc
from copy import copy

import torch


class SystemMatrix:
    """Abstract system matrix H with forward (H f) and backward (H^T g)."""

    def __init__(self, object_meta, proj_meta, obj2obj_transforms=None,
                 proj2proj_transforms=None) -> None:
        self.obj2obj_transforms = list(obj2obj_transforms or [])
        self.proj2proj_transforms = list(proj2proj_transforms or [])
        self.object_meta = object_meta
        self.proj_meta = proj_meta
        self.initialize_transforms()

    def __mul__(self, scalar):
        old_forward = copy(self.forward)
        old_backward = copy(self.backward)

        def new_forward(*args, **kwargs):
            return old_forward(*args, **kwargs) * scalar

        def new_backward(*args, **kwargs):
            return old_backward(*args, **kwargs) * scalar

        self.forward = new_forward
        self.backward = new_backward
        return self

    def __rmul__(self, scalar):
        return self.__mul__(scalar)

    def initialize_transforms(self) -> None:
        for t in self.obj2obj_transforms:
            t.configure(self.object_meta, self.proj_meta)
        for t in self.proj2proj_transforms:
            t.configure(self.object_meta, self.proj_meta)

    def _get_object_initial(self, device=None):
        import pytomography_gb300 as p
        return torch.ones(self.object_meta.shape).to(p.device if device is None else device)

    def _get_prior_FOV_scale(self):
        import pytomography_gb300 as p
        return torch.ones(self.object_meta.shape).to(p.device)

    @abc.abstractmethod
    def forward(self, object, **kwargs):
        ...

    @abc.abstractmethod
    def backward(self, proj, **kwargs):
        ...
