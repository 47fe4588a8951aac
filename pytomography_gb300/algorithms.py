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
        """Standard deviation of the counts m^T f_N in ``mask`` after sub-iteration N,
        from the iterates and predictions a ``DataStorageCallback`` stored (the method of
        preconditioned_gradient_ascent.py:170-215).

        Every sub-iteration is a map f_{n+1} = U_n(f_n, g).  The counts' sensitivity to
        the data is propagated backwards through the chain with the adjoint Jacobians of
        each stored step (``_StepJacobian``): a running object-space vector q starts at
        m (or the filtered mask), every step adds its data-space image J_g^T q to the
        projection-space sensitivity v, and q moves one step back as J_f^T q.  With
        Poisson data Var(m^T f_N) = sum_i g_i v_i^2 (plus the additive term's variance
        when requested).  Every operator application is projector calls on the GPU."""
        cb = data_storage_callback
        last = len(cb.objects) - 1 if subiteration_number is None else subiteration_number
        f_last = cb.objects[last].to(_p.device)
        q = mask.clone() if post_recon_filter is None else post_recon_filter(mask)
        if post_recon_filter is not None:
            f_last = post_recon_filter(f_last)
        v = None
        for n in reversed(range(last)):  # steps n -> n + 1, newest first
            step = _StepJacobian(self, cb, n)
            term = step.data_sensitivity(q, include_additive_term)
            v = term if v is None else v + term
            if n > 0:
                q = step.object_sensitivity(q)
        variance = torch.sum(v[0] * self.likelihood.projections * v[0])
        if include_additive_term:
            variance = variance + torch.sum(self.likelihood.additive_term_variance_estimate(v[1]))
        sd = torch.sqrt(variance).item()
        if not return_pct:
            return sd
        return sd, sd / (f_last * mask).sum().item() * 100

    def _uncertainty_subset(self, n: int):
        """Subset index sub-iteration n used (None without subsets)."""
        return None if self.n_subsets == 1 else n % self.n_subsets

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


class _StepJacobian:
    """Adjoint Jacobians of one stored sub-iteration of a linearly preconditioned update
    f_{n+1} = f_n + f_n c_n (grad L_n(f_n) - grad V(f_n)), clamped, where c_n is the
    algorithm's preconditioner factor for the step's subset.

    With D = diag(f_n c_n) and the likelihood's curvature blocks at the stored prediction
    (``PoissonCurvature``):
      object_sensitivity(q) = (L_ff - V_ff) D q + (f_{n+1} / (f_n + delta)) q
      data_sensitivity(q)   = [L_gf D q (, L_sf D q)] placed on the subset's projection
                              rows of full-size projection arrays.
    The ratio f_{n+1}/f_n stands for the derivative of the update's multiplicative part
    and, for clamped voxels, for the zero derivative of the clamp."""

    def __init__(self, alg, cb, n: int) -> None:
        self.alg = alg
        self.subset_idx = alg._uncertainty_subset(n)
        self.f = cb.objects[n].to(_p.device)
        self.f_next = cb.objects[n + 1].to(_p.device) if n + 1 < len(cb.objects) else None
        self.curv = alg.likelihood._curvature(self.f, cb.projections_predicted[n].to(_p.device),
                                              self.subset_idx)
        self.scale = self.f * alg._linear_preconditioner_factor(None, self.subset_idx)

    def object_sensitivity(self, q: torch.Tensor) -> torch.Tensor:
        dq = q * self.scale
        out = self.curv.ff(dq)
        prior = self.alg.prior
        if prior is not None:
            sm = self.alg.likelihood.system_matrix
            prior.set_beta_scale(sm.get_weighting_subset(self.subset_idx))
            prior.set_object(self.f)
            out = out - prior(derivative_order=2)(dq)
        return out + (self.f_next / (self.f + _p.delta)) * q

    def data_sensitivity(self, q: torch.Tensor, include_additive_term: bool) -> torch.Tensor:
        sm = self.alg.likelihood.system_matrix
        dq = q * self.scale
        parts = [self.curv.gf(dq)]
        if include_additive_term:
            parts.append(self.curv.sf(dq))
        full = tuple(sm.proj_meta.shape[-3:])
        out = torch.zeros((len(parts), *parts[0].shape[:-3], *full), device=parts[0].device)
        if self.subset_idx is None:
            rows = torch.arange(full[0], device=out.device)
        else:
            rows = sm.subset_indices_array[self.subset_idx].to(out.device)
        for k, p in enumerate(parts):
            out[k].index_copy_(out[k].dim() - 3, rows, p)
        return out


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

    def _callback_pairs(self):
        """(bed algorithm, callback) pairs for a list of per-bed callbacks, or
        [(None, callback)] for one callback that sees the stitched object."""
        cbs = self.callback
        if cbs is None:
            return []
        if isinstance(cbs, list):
            return list(zip(self.reconstruction_algorithms, cbs))
        return [(None, cbs)]

    def _multibed_callback(self, n_iter: int, n_subset: int) -> None:
        for alg, cb in self._callback_pairs():
            if alg is None:  # the stitched reconstruction
                self.object_prediction = cb.run(self.object_prediction, n_iter, n_subset)
            else:  # each bed's own iterate
                alg.callback = cb
                alg._compute_callback(n_iter=n_iter, n_subset=n_subset)

    def _finalize_callback(self) -> None:
        for alg, cb in self._callback_pairs():
            if alg is not None:
                alg.callback = cb
            cb.finalize(self.object_prediction if alg is None else alg.object_prediction)

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
