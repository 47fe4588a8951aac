"""SPECT metadata (src/pytomography/metadata/SPECT/spect_metadata.py:8-95)."""
from __future__ import annotations

from typing import Sequence

import torch

from ..geometry import compute_pad_size
from .metadata import ObjectMeta, ProjMeta


class SPECTObjectMeta(ObjectMeta):
    """Object-space metadata: voxel size ``dr`` (cm) and shape [Lx, Ly, Lz]."""

    def __init__(self, dr: list[float], shape: list[int]) -> None:
        self.dr = dr
        self.dx, self.dy, self.dz = dr[0], dr[1], dr[2]
        self.shape = shape
        self.compute_padded_shape()
        self.recon_method = None
        self.units = "counts"

    def compute_padded_shape(self) -> None:
        self.pad_size = compute_pad_size(self.shape[0])
        self.padded_shape = (int(self.shape[0] + 2 * self.pad_size),
                             int(self.shape[1] + 2 * self.pad_size), int(self.shape[2]))


class SPECTProjMeta(ProjMeta):
    """Projection metadata: detector angles (degrees) and radii (cm) per angle."""

    def __init__(self, projection_shape: Sequence, dr: list[float], angles: Sequence,
                 radii=None) -> None:
        self.angles = torch.tensor(angles).to(torch.float32)
        self.dr = dr
        self.radii = radii
        self.num_projections = len(angles)
        self.shape = (self.num_projections, projection_shape[0], projection_shape[1])
        self.compute_padded_shape()

    def compute_padded_shape(self) -> None:
        self.pad_size = compute_pad_size(self.shape[1])
        self.padded_shape = (int(self.shape[0]), int(self.shape[1] + 2 * self.pad_size),
                             int(self.shape[2]))


class StarGuideProjMeta(ProjMeta):
    """StarGuide projection metadata (metadata/SPECT/starguide_metadata.py:5-34):
    projection shape (n, window width, nz); per projection its angle (degrees),
    acquisition time (ms), offset of the detector along y (cm) and radius (cm, for the
    PSF)."""

    def __init__(self, projection_shape: Sequence, angles: Sequence, times=None, offsets=None,
                 radii: Sequence | None = None) -> None:
        self.angles = angles
        self.radii = radii
        self.offsets = offsets
        self.times = times
        self.num_projections = len(angles)
        self.shape = projection_shape


class SPECTPSFMeta:
    """Depth-dependent PSF: sigma(d) = sigma_fit(d, *params) (cm)."""

    def __init__(self, sigma_fit_params: Sequence[float],
                 sigma_fit=lambda r, a, b: a * r + b, kernel_dimensions: str = "2D",
                 min_sigmas: float | None = 3, shape: str = "gaussian") -> None:
        self.sigma_fit_params = sigma_fit_params
        self.sigma_fit = sigma_fit
        self.kernel_dimensions = kernel_dimensions
        self.min_sigmas = 1 if shape == "square" else min_sigmas
        self.shape = shape

    def __repr__(self):
        attrs = [f"{a} = {getattr(self, a)}\n" for a in dir(self)
                 if not callable(getattr(self, a)) and not a.startswith("__")]
        return "".join(attrs)
