"""OSEM / BSREM update loop.

Mirror of ``PreconditionedGradientAscentAlgorithm.__call__``, ``OSEM`` and ``BSREM``
(src/pytomography/algorithms/preconditioned_gradient_ascent.py:14-129, 301-329, 436-474).

Two execution forms share the loop:

* ``fused=True`` (default when the system matrix is this package's
  ``SPECTSystemMatrix`` and the likelihood is ``PoissonLogLikelihood``): each
  sub-iteration is one C-ABI call (``gb_spect_osem_step`` / ``gb_spect_bsrem_step``):
  forward kernel with the g/(Hf+s+delta) epilogue, back-projection kernels, and the
  preconditioned update (and, for BSREM, the RDP gradient) fused into the last one.
* ``fused=False``: the reference's own sequence of forward, torch elementwise ratio,
  backward and torch elementwise update ("plain" per-call path).
"""
from __future__ import annotations

from collections.abc import Callable

import torch

import pytomography_gb300 as _p

from .likelihoods import PoissonLogLikelihood


class PreconditionedGradientAscentAlgorithm:
    def __init__(self, likelihood, prior=None, object_initial: torch.Tensor | None = None,
                 addition_after_iteration: float = 0, fused: bool | None = None, **kwargs) -> None:
        self.likelihood = likelihood
        if object_initial is None:
            self.object_prediction = likelihood.system_matrix._get_object_initial(_p.device)
        else:
            self.object_prediction = object_initial.to(_p.device).to(_p.dtype)
        self.prior = prior
        if self.prior is not None:
            self.prior.set_object_meta(likelihood.system_matrix.object_meta)
            self.prior.set_FOV_scale(likelihood.system_matrix._get_prior_FOV_scale())
        self.objects_stored = []
        self.projections_predicted_stored = []
        self.addition_after_iteration = addition_after_iteration
        self._fused_request = fused

    def _set_n_subsets(self, n_subsets: int) -> None:
        self.n_subsets = n_subsets
        self.likelihood._set_n_subsets(n_subsets)

    def _compute_preconditioner(self, object, n_iter, n_subset):
        raise NotImplementedError

    def _compute_callback(self, n_iter: int, n_subset: int) -> None:
        self.object_prediction = self.callback.run(self.object_prediction, n_iter, n_subset)

    def _can_fuse(self) -> bool:
        from .projectors.PET import PETLMSystemMatrix
        from .projectors.SPECT import SPECTSystemMatrix
        sm = self.likelihood.system_matrix
        kind = self._fused_kind()
        ok = (type(self.likelihood) is PoissonLogLikelihood and kind is not None
              and (isinstance(sm, SPECTSystemMatrix)
                   or (isinstance(sm, PETLMSystemMatrix) and kind == "osem"
                       and not sm.scale_projection_by_sensitivity
                       and not sm.obj2obj_transforms
                       and sm.output_device == sm.device)))
        if self._fused_request is True and not ok:
            raise NotImplementedError("this likelihood / system matrix / prior has no fused step")
        return ok if self._fused_request is None else bool(self._fused_request)

    def _fused_kind(self):
        return None

    # ------------------------------------------------------------ uncertainty
    def compute_uncertainty(self, mask: torch.Tensor, data_storage_callback,
                            subiteration_number: int | None = None, return_pct: bool = False,
                            include_additive_term: bool = False, post_recon_filter=None):
        """Uncertainty of the sum of counts in ``mask`` from the iterates stored by a
        ``DataStorageCallback`` (preconditioned_gradient_ascent.py:170-215): the
        variance propagates back through every sub-iteration with the operators Q and B,
        whose projector calls run on the GPU kernels."""
        cb = data_storage_callback
        if subiteration_number is None:
            subiteration_number = len(cb.objects) - 1
        final_recon = cb.objects[subiteration_number].to(_p.device)
        if post_recon_filter is not None:
            Q = post_recon_filter(mask)
            final_recon = post_recon_filter(final_recon)
        else:
            Q = mask.clone()
        V = 0
        for n in range(subiteration_number, 0, -1):
            V = V + self._compute_B(Q, cb, n - 1, include_additive_term=include_additive_term)
            if n > 1:
                Q = self._compute_Q(Q, cb, n - 1)
        abs2 = torch.sum(V[0] * self.likelihood.projections * V[0])
        if include_additive_term:
            abs2 = abs2 + torch.sum(self.likelihood.additive_term_variance_estimate(V[1]))
        unc_abs = torch.sqrt(abs2).item()
        if not return_pct:
            return unc_abs
        return unc_abs, unc_abs / (final_recon * mask).sum().item() * 100

    def _uncertainty_subset(self, n: int):
        return None if self.n_subsets == 1 else n % self.n_subsets

    def _compute_Q(self, input, cb, n: int):
        """Q of the uncertainty recursion (preconditioned_gradient_ascent.py:217-251)."""
        subset_idx = self._uncertainty_subset(n)
        f_n = cb.objects[n].to(_p.device)
        f_next = cb.objects[n + 1].to(_p.device)
        fp_n = cb.projections_predicted[n].to(_p.device)
        grad_ff = self.likelihood.compute_gradient_ff(f_n, fp_n, subset_idx)
        out = input * f_n * self._linear_preconditioner_factor(None, subset_idx)
        if self.prior is not None:
            self.prior.set_beta_scale(self.likelihood.system_matrix.get_weighting_subset(subset_idx))
            self.prior.set_object(f_n)
            out = grad_ff(out) - self.prior(derivative_order=2)(out)
        else:
            out = grad_ff(out)
        return out + (f_next / (f_n + _p.delta)) * input

    def _compute_B(self, input, cb, n: int, include_additive_term: bool = False):
        """B of the uncertainty recursion (preconditioned_gradient_ascent.py:253-299)."""
        sm = self.likelihood.system_matrix
        subset_idx = self._uncertainty_subset(n)
        if subset_idx is None:
            rows = torch.arange(sm.proj_meta.shape[0]).to(torch.long).to(_p.device)
        else:
            rows = sm.subset_indices_array[subset_idx]
        f_n = cb.objects[n].to(_p.device)
        fp_n = cb.projections_predicted[n].to(_p.device)
        out = input * f_n * self._linear_preconditioner_factor(None, subset_idx)
        primary = self.likelihood.compute_gradient_gf(f_n, fp_n, subset_idx)(out)
        n_out = 2 if include_additive_term else 1
        total = torch.zeros((n_out, *fp_n.shape[:-3], *sm.proj_meta.shape[-3:]),
                            device=primary.device)
        total[0, ..., rows, :, :] = primary
        if include_additive_term:
            total[1, ..., rows, :, :] = self.likelihood.compute_gradient_sf(f_n, fp_n,
                                                                            subset_idx)(out)
        return total

    def _fused_begin(self) -> None:
        pass

    def _fused_step(self, j: int, subset_idx):
        raise NotImplementedError

    def __call__(self, n_iters: int, n_subsets: int = 1, n_subset_specific: int | None = None,
                 callback=None):
        self.callback = callback
        self.n_iters = n_iters
        self._set_n_subsets(n_subsets)
        fused = self._can_fuse()
        if fused:
            self.object_prediction = self.object_prediction.to(torch.float32).contiguous()
            self._fused_begin()
        for j in range(n_iters):
            for k in range(n_subsets):
                if n_subset_specific is not None and n_subset_specific != k:
                    continue
                subset_idx = None if n_subsets == 1 else k
                if fused:
                    self._fused_step(j, subset_idx)
                else:
                    if bool(self.prior):
                        self.prior.set_object(torch.clone(self.object_prediction).to(_p.device))
                        self.prior.set_beta_scale(
                            self.likelihood.system_matrix.get_weighting_subset(subset_idx))
                        self.prior_gradient = self.prior(derivative_order=1)
                    else:
                        self.prior_gradient = 0
                    grad = self.likelihood.compute_gradient(self.object_prediction, subset_idx)
                    pre = self._compute_preconditioner(self.object_prediction, j, subset_idx)
                    self.object_prediction += pre * (grad - self.prior_gradient)
                    self.object_prediction[self.object_prediction <= self.addition_after_iteration] = \
                        self.addition_after_iteration
                if self.callback is not None:
                    self._compute_callback(n_iter=j, n_subset=k)
        if self.callback is not None:
            self.callback.finalize(self.object_prediction)
        return self.object_prediction


class LinearPreconditionedGradientAscentAlgorithm(PreconditionedGradientAscentAlgorithm):
    def _linear_preconditioner_factor(self, n_iter: int, n_subset: int):
        raise NotImplementedError

    def _compute_preconditioner(self, object, n_iter, n_subset):
        return object * self._linear_preconditioner_factor(n_iter, n_subset)


class OSEM(LinearPreconditionedGradientAscentAlgorithm):
    """f <- f + f / H_m^T 1 * grad L."""

    def __init__(self, likelihood, object_initial: torch.Tensor | None = None,
                 fused: bool | None = None) -> None:
        super().__init__(likelihood=likelihood, object_initial=object_initial, fused=fused)

    def _linear_preconditioner_factor(self, n_iter, n_subset):
        return 1 / (self.likelihood._get_normBP(n_subset) + _p.delta)

    def _fused_kind(self):
        return "osem"

    def _fused_step(self, j, subset_idx):
        lik = self.likelihood
        sm = lik.system_matrix
        from .projectors.PET import PETLMSystemMatrix
        if isinstance(sm, PETLMSystemMatrix):
            s = lik.additive_term if lik.exists_additive_term else None
            sm.osem_step(self.object_prediction, lik.projections, s,
                         lik._get_normBP(subset_idx), subset_idx)
            return
        n_sel = sm._n_sel(subset_idx)
        pred = getattr(self, "_pred_buf", None)
        if pred is None or pred.shape[0] != n_sel:
            pred = torch.empty((n_sel, *sm.proj_meta.shape[1:]), device=sm.device)
            self._pred_buf = pred
        s = lik.additive_term if lik.exists_additive_term else None
        sm.osem_step(self.object_prediction, lik.projections, s, lik._get_normBP(subset_idx),
                     subset_idx, predicted=pred)
        lik.projections_predicted = pred


class BSREM(LinearPreconditionedGradientAscentAlgorithm):
    """f <- f + alpha(n) f / (w_m sum_k H_k^T 1) * (grad L - grad V), floor 1e-4."""

    def __init__(self, likelihood, object_initial: torch.Tensor | None = None, prior=None,
                 relaxation_sequence: Callable = lambda _: 1, addition_after_iteration=1e-4,
                 fused: bool | None = None) -> None:
        self.relaxation_sequence = relaxation_sequence
        super().__init__(likelihood=likelihood, object_initial=object_initial, prior=prior,
                         addition_after_iteration=addition_after_iteration, fused=fused)

    def _linear_preconditioner_factor(self, n_iter, n_subset):
        relaxation_factor = self.relaxation_sequence(n_iter)
        norm_BP = self.likelihood._get_normBP(n_subset, return_sum=True)
        w = self.likelihood.system_matrix.get_weighting_subset(n_subset)
        return relaxation_factor / (w * norm_BP + _p.delta)

    def _fused_kind(self):
        from .priors import RelativeDifferencePrior
        if getattr(getattr(self, "callback", None), "needs_projections_predicted", False):
            return None  # the fused BSREM step keeps its predicted projections inside
        if self.prior is None or isinstance(self.prior, RelativeDifferencePrior):
            return "bsrem"
        return None

    def _fused_begin(self) -> None:
        lik = self.likelihood
        self._nbp_sum = lik._get_normBP(None if self.n_subsets == 1 else 0,
                                        return_sum=True).contiguous()

    def _fused_step(self, j, subset_idx):
        lik = self.likelihood
        sm = lik.system_matrix
        out = getattr(self, "_pingpong", None)
        if out is None or out.shape != self.object_prediction.shape:
            out = torch.empty_like(self.object_prediction)
        s = lik.additive_term if lik.exists_additive_term else None
        sm.bsrem_step(self.object_prediction, out, lik.projections, s,
                      lik._get_normBP(subset_idx).contiguous(), self._nbp_sum,
                      float(self.relaxation_sequence(j)), float(sm.get_weighting_subset(subset_idx)),
                      prior=self.prior, floor_value=float(self.addition_after_iteration),
                      subset_idx=subset_idx)
        self._pingpong = self.object_prediction
        self.object_prediction = out


class PGAAMultiBedSPECT(PreconditionedGradientAscentAlgorithm):
    """Multi-bed SPECT: one reconstruction algorithm per bed position, sub-iteration by
    sub-iteration, stitched after every sub-iteration (preconditioned_gradient_ascent.py:
    550-663).

    ``files_NM`` of the reference are DICOM files whose headers give each bed's z
    position; here pass the z positions (``bed_z``, any length unit) and the slice spacing
    in the same unit.  When every bed runs fused OSEM on a SPECT system matrix and no
    callback is given, the beds' sub-iterations run together as CUDA graphs
    (``BatchedOSEM``); the iterates are the same as bed by bed.
    """

    def __init__(self, bed_z, reconstruction_algorithms, slice_spacing: float | None = None,
                 batched: bool = True) -> None:
        if any(isinstance(b, str) for b in bed_z):
            raise NotImplementedError("DICOM headers are not read here: pass the beds' z "
                                      "positions and slice_spacing")
        if slice_spacing is None:
            raise ValueError("slice_spacing is required with explicit bed positions")
        self.bed_z = [float(b) for b in bed_z]
        self.slice_spacing = float(slice_spacing)
        self.reconstruction_algorithms = list(reconstruction_algorithms)
        self.batched = batched

    def _stitch(self, recons):
        from .io.SPECT import stitch_multibed
        return stitch_multibed(torch.stack(recons), self.bed_z, self.slice_spacing)

    def _batch(self, n_subsets):
        from .batched import BatchedOSEM
        from .projectors.SPECT import SPECTSystemMatrix
        algs = self.reconstruction_algorithms
        ok = self.batched and all(
            type(a) is OSEM and a._fused_request is not False
            and type(a.likelihood) is PoissonLogLikelihood
            and isinstance(a.likelihood.system_matrix, SPECTSystemMatrix) for a in algs)
        if not ok:
            return None
        return BatchedOSEM([a.likelihood for a in algs], n_subsets=n_subsets,
                           object_initial=[a.object_prediction for a in algs])

    def __call__(self, n_iters: int, n_subsets: int, callback=None) -> torch.Tensor:
        self.callback = callback
        batch = self._batch(n_subsets) if callback is None else None
        for i in range(n_iters):
            for j in range(n_subsets):
                if batch is not None:
                    batch.step(j)
                    self.recons = batch.objects
                else:
                    self.recons = [a(1, n_subsets, n_subset_specific=j)
                                   for a in self.reconstruction_algorithms]
                self.object_prediction = self._stitch(self.recons)
                self._multibed_callback(i, j)
        if batch is not None:
            for a, f in zip(self.reconstruction_algorithms, batch.objects):
                a.object_prediction = f.clone()
        self._finalize_callback()
        return self.object_prediction

    def _multibed_callback(self, n_iter: int, n_subset: int) -> None:
        if self.callback is None:
            return
        if isinstance(self.callback, list):
            for a, cb in zip(self.reconstruction_algorithms, self.callback):
                a.callback = cb
                a._compute_callback(n_iter=n_iter, n_subset=n_subset)
        else:
            self.object_prediction = self.callback.run(self.object_prediction, n_iter, n_subset)

    def _finalize_callback(self) -> None:
        if self.callback is None:
            return
        if isinstance(self.callback, list):
            for a, cb in zip(self.reconstruction_algorithms, self.callback):
                a.callback = cb
                cb.finalize(a.object_prediction)
        else:
            self.callback.finalize(self.object_prediction)

    def compute_uncertainty(self, mask: torch.Tensor, data_storage_callbacks,
                            subiteration_number: int | None = None, return_pct: bool = False,
                            include_additive_term: bool = False):
        """Uncertainty of the counts in ``mask`` (stitched-image shape): each bed's share
        of the mask, weighted by that bed's own stitching weights, goes through the bed's
        ``compute_uncertainty`` and the results add in quadrature
        (preconditioned_gradient_ascent.py:623-663).  The reference weights every bed with
        the first bed's profile (its stitching helper concatenates the weights instead of
        stacking them); each bed's own weights are used here."""
        from .io.SPECT import stitch_multibed
        if subiteration_number is None:
            subiteration_number = len(data_storage_callbacks[0].objects) - 1
        recons = [cb.objects[subiteration_number].to(_p.device) for cb in data_storage_callbacks]
        weights, zs = stitch_multibed(torch.stack(recons), self.bed_z, self.slice_spacing,
                                      return_stitching_weights=True)
        unc, total = [], 0.0
        lz = recons[0].shape[-1]
        for k in range(len(recons)):
            mask_k = mask[:, :, zs[k]:zs[k] + lz] * weights[k]
            if mask_k.sum() == 0:
                continue
            unc.append(self.reconstruction_algorithms[k].compute_uncertainty(
                mask_k, data_storage_callbacks[k], subiteration_number, return_pct=False,
                include_additive_term=include_additive_term))
            total += (recons[k] * mask_k).sum().item()
        unc_abs = torch.sqrt(torch.sum(torch.tensor(unc) ** 2)).item()
        if return_pct:
            return unc_abs, unc_abs / total * 100
        return unc_abs
