"""Poisson likelihood of the projector path.

Interface mirror of ``Likelihood`` / ``PoissonLogLikelihood``
(src/pytomography/likelihoods/likelihood.py:8-91, poisson_log_likelihood.py:8-128): the
same class names, constructor arguments, method names and return conventions, so the
reconstruction loops and the uncertainty estimate call it unchanged.

With predicted counts y(f) = H f + s, data g and delta = ``pytomography_gb300.delta``:

* log-likelihood  L(f) = sum_i g_i log y_i - y_i;
* subset gradient grad_m L = H_m^T (g_m / (y_m + delta)) - H_m^T 1;
* the second-order blocks the uncertainty recursion needs, linearised at a stored
  prediction y (``PoissonCurvature``):
  ff: x -> -H^T diag(g / (y^2 + delta)) H x  (object -> object),
  gf: x -> diag(1 / (y + delta)) H x          (object -> data),
  sf: x -> -diag(g / (y + delta)^2) H x       (object -> additive term).
"""
from __future__ import annotations

from typing import Callable

import torch

import pytomography_gb300 as _p


class Likelihood:
    """Data term of a reconstruction: the system matrix, the measured projections and the
    additive term, plus the normalisation images H_m^T 1 of the current subset split.

    Listmode system matrices take no projections (every event counts once); the data is
    then the one-element tensor [1.]."""

    def __init__(self, system_matrix, projections: torch.Tensor | None = None,
                 additive_term: torch.Tensor | None = None,
                 additive_term_variance_estimate: Callable | None = None) -> None:
        self.system_matrix = system_matrix
        self.projections = (torch.ones(1, device=_p.device) if projections is None
                            else projections)
        data = self.projections
        self.exists_additive_term = isinstance(additive_term, torch.Tensor)
        if self.exists_additive_term:
            self.additive_term = additive_term.to(data.device, _p.dtype)
        else:
            self.additive_term = torch.zeros(data.shape, device=data.device, dtype=_p.dtype)
        self.additive_term_variance_estimate = additive_term_variance_estimate
        self.n_subsets = None
        self._normalisation_split = None  # subset count the stored H_m^T 1 belong to

    # ------------------------------------------------------------ normalisation
    def _set_n_subsets(self, n_subsets: int) -> None:
        """Split the data into ``n_subsets`` and keep every subset's H_m^T 1 (one back
        projection of ones per subset, recomputed only when the split changes)."""
        sm = self.system_matrix
        self.n_subsets = n_subsets
        if n_subsets < 2:
            self.norm_BP = sm.compute_normalization_factor()
        else:
            sm.set_n_subsets(n_subsets)
            if self._normalisation_split != n_subsets:
                if hasattr(sm, "compute_normalization_factors"):
                    self.norm_BPs = sm.compute_normalization_factors()
                else:
                    self.norm_BPs = [sm.compute_normalization_factor(k) for k in range(n_subsets)]
        self._normalisation_split = n_subsets

    def _get_normBP(self, subset_idx, return_sum: bool = False):
        """H_m^T 1 of one subset, or with ``return_sum`` the sum over all subsets (the
        full normalisation sum_k H_k^T 1 that BSREM's preconditioner uses)."""
        if subset_idx is None:
            return self.norm_BP
        if return_sum:
            total = self.norm_BPs[0].clone()
            for nb in self.norm_BPs[1:]:
                total += nb
            return total
        return self.norm_BPs[subset_idx].to(_p.device)

    def _get_projection_subset(self, projections, subset_idx=None):
        return projections if subset_idx is None else \
            self.system_matrix.get_projection_subset(projections, subset_idx)

    def compute_gradient(self, *args, **kwargs):
        raise NotImplementedError("Compute gradient not implemented for this likelihood function")


class PoissonCurvature:
    """Second-order blocks of the Poisson log-likelihood of one subset, linearised at a
    prediction ``predicted`` = H_m f + s_m (see the module docstring).  Each block is one
    forward projection plus elementwise work (plus one back projection for ff)."""

    def __init__(self, likelihood: "PoissonLogLikelihood", subset_idx, predicted: torch.Tensor):
        self.H = likelihood.system_matrix
        self.subset_idx = subset_idx
        self.g = likelihood._get_projection_subset(likelihood.projections, subset_idx)
        self.y = predicted

    def _project(self, x: torch.Tensor) -> torch.Tensor:
        return self.H.forward(x, self.subset_idx)

    def ff(self, x: torch.Tensor) -> torch.Tensor:
        weight = self.g / (self.y ** 2 + _p.delta)
        return -self.H.backward(self._project(x) * weight, self.subset_idx)

    def gf(self, x: torch.Tensor) -> torch.Tensor:
        return self._project(x) / (self.y + _p.delta)

    def sf(self, x: torch.Tensor) -> torch.Tensor:
        return -self._project(x) * self.g / (self.y + _p.delta) ** 2


class PoissonLogLikelihood(Likelihood):
    """L(g|f) = sum_i g_i ln([Hf]_i + s_i) - [Hf]_i - s_i."""

    def compute_gradient(self, object: torch.Tensor, subset_idx: int | None = None,
                         norm_BP_subset_method: str = "subset_specific") -> torch.Tensor:
        """grad_m L(f) = H_m^T (g_m / (H_m f + s_m + delta)) - H_m^T 1; keeps the
        prediction H_m f + s_m in ``projections_predicted``."""
        H = self.system_matrix
        g_m = self._get_projection_subset(self.projections, subset_idx)
        s_m = self._get_projection_subset(self.additive_term, subset_idx)
        predicted = H.forward(object, subset_idx) + s_m
        self.projections_predicted = predicted
        ratio = g_m / (predicted + _p.delta)
        return H.backward(ratio, subset_idx) - self._get_normBP(subset_idx)

    def _curvature(self, object, predicted, subset_idx) -> PoissonCurvature:
        if predicted is None:
            predicted = self.system_matrix.forward(object, subset_idx)
        return PoissonCurvature(self, subset_idx, predicted)

    def compute_gradient_ff(self, object, precomputed_forward_projection=None, subset_idx=None):
        """Operator x -> (d^2 L / df^2) x at ``object`` (or at the given prediction)."""
        return self._curvature(object, precomputed_forward_projection, subset_idx).ff

    def compute_gradient_gf(self, object, precomputed_forward_projection=None, subset_idx=None):
        """Operator x -> (d^2 L / dg df) x."""
        return self._curvature(object, precomputed_forward_projection, subset_idx).gf

    def compute_gradient_sf(self, object, precomputed_forward_projection=None, subset_idx=None):
        """Operator x -> (d^2 L / ds df) x."""
        return self._curvature(object, precomputed_forward_projection, subset_idx).sf
