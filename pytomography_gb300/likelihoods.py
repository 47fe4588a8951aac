"""Likelihood mirrors (src/pytomography/likelihoods/likelihood.py:8-139,
poisson_log_likelihood.py:8-128)."""
from __future__ import annotations

from typing import Callable

import torch

import pytomography_gb300 as _p


class Likelihood:
    """Subset bookkeeping and cached normalisation back projections H_m^T 1."""

    def __init__(self, system_matrix, projections: torch.Tensor | None = None,
                 additive_term: torch.Tensor | None = None,
                 additive_term_variance_estimate: Callable | None = None) -> None:
        self.system_matrix = system_matrix
        if projections is None:  # listmode reconstruction
            self.projections = torch.tensor([1.0]).to(_p.device)
        else:
            self.projections = projections
        self.FP = None
        if isinstance(additive_term, torch.Tensor):
            self.additive_term = additive_term.to(self.projections.device).to(_p.dtype)
            self.exists_additive_term = True
        else:
            self.additive_term = torch.zeros(self.projections.shape).to(
                self.projections.device).to(_p.dtype)
            self.exists_additive_term = False
        self.n_subsets_previous = -1
        self.additive_term_variance_estimate = additive_term_variance_estimate

    def _set_n_subsets(self, n_subsets: int) -> None:
        self.n_subsets = n_subsets
        if n_subsets < 2:
            self.norm_BP = self.system_matrix.compute_normalization_factor()
        else:
            self.system_matrix.set_n_subsets(n_subsets)
            if self.n_subsets_previous != self.n_subsets:
                self.norm_BPs = [self.system_matrix.compute_normalization_factor(k)
                                 for k in range(self.n_subsets)]
        self.n_subsets_previous = n_subsets

    def _get_projection_subset(self, projections, subset_idx=None):
        if subset_idx is None:
            return projections
        return self.system_matrix.get_projection_subset(projections, subset_idx)

    def _get_normBP(self, subset_idx, return_sum: bool = False):
        if subset_idx is None:
            return self.norm_BP
        if return_sum:
            return torch.stack(self.norm_BPs).sum(axis=0)
        return self.norm_BPs[subset_idx].to(_p.device)

    def compute_gradient(self, *args, **kwargs):
        raise NotImplementedError("Compute gradient not implemented for this likelihood function")


class PoissonLogLikelihood(Likelihood):
    """L(g|f) = sum_i g_i ln([Hf]_i + s_i) - [Hf]_i - s_i."""

    def compute_gradient(self, object: torch.Tensor, subset_idx: int | None = None,
                         norm_BP_subset_method: str = "subset_specific") -> torch.Tensor:
        proj_subset = self._get_projection_subset(self.projections, subset_idx)
        additive_subset = self._get_projection_subset(self.additive_term, subset_idx)
        self.projections_predicted = self.system_matrix.forward(object, subset_idx) + additive_subset
        norm_BP = self._get_normBP(subset_idx)
        return self.system_matrix.backward(proj_subset / (self.projections_predicted + _p.delta),
                                           subset_idx) - norm_BP

    def compute_gradient_ff(self, object, precomputed_forward_projection=None, subset_idx=None):
        FP = self.system_matrix.forward(object, subset_idx) \
            if precomputed_forward_projection is None else precomputed_forward_projection
        proj_subset = self._get_projection_subset(self.projections, subset_idx)

        def operator(input):
            input = self.system_matrix.forward(input, subset_idx)
            input = input * proj_subset / (FP ** 2 + _p.delta)
            return -self.system_matrix.backward(input, subset_idx)
        return operator

    def compute_gradient_gf(self, object, precomputed_forward_projection=None, subset_idx=None):
        FP = self.system_matrix.forward(object, subset_idx) \
            if precomputed_forward_projection is None else precomputed_forward_projection

        def operator(input):
            input = self.system_matrix.forward(input, subset_idx)
            return input / (FP + _p.delta)
        return operator

    def compute_gradient_sf(self, object, precomputed_forward_projection=None, subset_idx=None):
        proj_subset = self._get_projection_subset(self.projections, subset_idx)
        FP = self.system_matrix.forward(object, subset_idx) \
            if precomputed_forward_projection is None else precomputed_forward_projection

        def operator(input):
            input = self.system_matrix.forward(input, subset_idx)
            return -input * proj_subset / (FP + _p.delta) ** 2
        return operator
