"""``KEMSystemMatrix`` (src/pytomography/projectors/shared/kem_system_matrix.py:4-59): the
system matrix H K of a kernel-method reconstruction, forward H (K alpha) and backward
K^T (H^T g), with the normalisation K^T H_m^T 1."""
from __future__ import annotations

from .system_matrix import SystemMatrix


class KEMSystemMatrix(SystemMatrix):
    def __init__(self, system_matrix, kem_transform) -> None:
        self.object_meta = system_matrix.object_meta
        self.proj_meta = system_matrix.proj_meta
        self.obj2obj_transforms = []
        self.proj2proj_transforms = []
        self.system_matrix = system_matrix
        self.kem_transform = kem_transform
        self.kem_transform.configure(system_matrix.object_meta, system_matrix.proj_meta)
        self.set_n_subsets = self.system_matrix.set_n_subsets
        self.get_projection_subset = self.system_matrix.get_projection_subset
        # the reference binds get_projection_subset here (kem_system_matrix.py:22), which
        # breaks subset-weighted priors; the subset weighting is the wrapped matrix's
        self.get_weighting_subset = self.system_matrix.get_weighting_subset

    @property
    def subset_indices_array(self):
        return self.system_matrix.subset_indices_array

    def compute_normalization_factor(self, subset_idx: int | None = None):
        return self.kem_transform.backward(
            self.system_matrix.compute_normalization_factor(subset_idx))

    def forward(self, object, subset_idx=None):
        return self.system_matrix.forward(self.kem_transform.forward(object), subset_idx)

    def backward(self, proj, subset_idx=None):
        return self.kem_transform.backward(self.system_matrix.backward(proj, subset_idx))

    def _get_object_initial(self, device=None):
        return self.system_matrix._get_object_initial(device)

    def _get_prior_FOV_scale(self):
        return self.system_matrix._get_prior_FOV_scale()
