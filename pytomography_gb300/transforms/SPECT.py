"""SPECT obj2obj plugins: attenuation and depth-dependent Gaussian PSF.

Mirrors of ``SPECTAttenuationTransform`` (src/pytomography/transforms/SPECT/attenuation.py:24-115)
and ``SPECTPSFTransform`` (src/pytomography/transforms/SPECT/psf.py:101-231).  They carry
configuration; ``SPECTSystemMatrix`` lowers them into its fused CUDA plan, where the
attenuation factor and the per-plane blur run inside the projector kernels.  The
per-angle plugin calls (``forward(object_i, ang_idx)``) exist only inside that fused
path and raise when called on their own.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import geometry
from .transform import Transform


class SPECTAttenuationTransform(Transform):
    """Attenuation plugin: exp(-rev_cumsum(mu_rot * dx)) towards the detector at +x."""

    def __init__(self, attenuation_map: torch.Tensor | None = None, filepath=None,
                 mode: str = "constant", assume_padded: bool = True,
                 HU2mu_technique="from_table") -> None:
        super().__init__()
        if filepath is not None:
            raise NotImplementedError("CT DICOM loading is outside the projector hot path; "
                                      "pass attenuation_map")
        if attenuation_map is None:
            raise Exception("Please supply only one of `attenuation_map` or `filepath` as arguments")
        # assume_padded=False: the attenuation map is rotated in the unpadded frame, as the
        # StarGuide system matrix needs (attenuation.py:85-89)
        self.attenuation_map = attenuation_map
        self.mode = mode
        self.assume_padded = assume_padded

    def forward(self, object_i, ang_idx):
        raise NotImplementedError("applied inside SPECTSystemMatrix's fused projector")

    def backward(self, object_i, ang_idx):
        raise NotImplementedError("applied inside SPECTSystemMatrix's fused projector")


class SPECTPSFTransform(Transform):
    """Depth-dependent separable PSF plugin (Gaussian or square per-plane kernels)."""

    def __init__(self, psf_meta=None, psf_operator=None, assume_padded: bool = True) -> None:
        super().__init__()
        if psf_operator is not None:
            raise NotImplementedError("a user psf_operator network cannot be fused; "
                                      "use psf_meta")
        self.psf_meta = psf_meta
        self.psf_operator = None
        self.assume_padded = assume_padded

    def configure(self, object_meta, proj_meta) -> None:
        super().configure(object_meta, proj_meta)
        self._configure_tables()

    def _get_sigma(self, radius: float) -> np.ndarray:
        """Per-plane sigma over the padded x extent, or the unpadded one with
        assume_padded=False (psf.py:172-197)."""
        dim = self.object_meta.shape[0]
        if self.assume_padded:
            dim += 2 * geometry.compute_pad_size(self.object_meta.shape[0])
        return geometry.psf_sigma(dim, radius, self.object_meta.dx, self.psf_meta)

    def _compute_kernel_size(self, radius, axis) -> int:
        return geometry.psf_kernel_size(self._get_sigma(radius), self.object_meta.dr[axis],
                                        self.psf_meta.min_sigmas)

    def _configure_tables(self) -> None:
        """Per unique radius: taps along r (y) and z for every padded plane
        (psf.py:119-142)."""
        self.radii_unique = [float(r) for r in np.unique(self.proj_meta.radii)]
        self.tables = {}
        for radius in self.radii_unique:
            kr = self._compute_kernel_size(radius, 0)
            kz = self._compute_kernel_size(radius, 2)
            sigma = self._get_sigma(radius)
            wr = geometry.psf_taps(sigma / self.object_meta.dx, kr, self.psf_meta.shape)
            wz = geometry.psf_taps(sigma / self.object_meta.dz, kz, self.psf_meta.shape)
            two_d = self.psf_meta.kernel_dimensions == "2D"
            self.tables[radius] = (wr, wz if two_d else None)

    def forward(self, object, ang_idx):
        raise NotImplementedError("applied inside SPECTSystemMatrix's fused projector")

    def backward(self, object, ang_idx):
        raise NotImplementedError("applied inside SPECTSystemMatrix's fused projector")
