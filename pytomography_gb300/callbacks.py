"""Reconstruction callbacks (src/pytomography/callbacks/callback.py,
callbacks/data_saving.py).

``DataStorageCallback`` keeps, for every sub-iteration, the object before the update and
the predicted projections H_m f + s_m the update used; ``compute_uncertainty`` of the
reconstruction algorithms walks these back.  The fused OSEM step writes its predicted
projections for it; BSREM with this callback runs the plain per-call sequence.
"""
from __future__ import annotations

import torch


class Callback:
    """Hook run after every sub-iteration; ``run`` may return a modified object."""

    def run(self, object: torch.Tensor, n_iter: int, n_subset: int) -> torch.Tensor:
        return object

    def finalize(self, object: torch.Tensor) -> None:
        pass


class DataStorageCallback(Callback):
    needs_projections_predicted = True

    def __init__(self, likelihood, object_initial: torch.Tensor) -> None:
        self.object_previous = torch.clone(object_initial)
        self.objects = []
        self.projections_predicted = []
        self.likelihood = likelihood

    def run(self, object: torch.Tensor, n_iter: int, n_subset: int) -> torch.Tensor:
        self.objects.append(self.object_previous.cpu())
        self.projections_predicted.append(self.likelihood.projections_predicted.cpu())
        self.object_previous = torch.clone(object)
        return object

    def finalize(self, object: torch.Tensor) -> None:
        self.objects.append(object.cpu())
        self.projections_predicted.append(None)
