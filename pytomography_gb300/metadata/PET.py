"""PET listmode metadata mirrors.

``PETTOFMeta`` (src/pytomography/metadata/PET/pet_tof_metadata.py:5-37),
``PETLMProjMeta`` (src/pytomography/metadata/PET/petlm_metadata.py:6-39) and the scanner
lookup table builder ``get_scanner_LUT`` (src/pytomography/io/PET/shared.py:275-396).
"""
from __future__ import annotations

import numpy as np
import torch


class PETTOFMeta:
    """TOF binning: num_bins over tof_range (mm), Gaussian FWHM (mm)."""

    def __init__(self, num_bins: int, tof_range: float, fwhm: float, n_sigmas: float = 3,
                 bin_type: str = "symmetric"):
        tof_bin_edges = torch.linspace(-1, 1, num_bins + 1) * tof_range / 2
        bin_width = tof_bin_edges[1] - tof_bin_edges[0]
        self.num_bins = num_bins
        self.bin_width = bin_width
        self.sigma = torch.tensor([fwhm / 2.355], dtype=torch.float32)
        self.n_sigmas = n_sigmas
        self.bin_edges = tof_bin_edges
        self.bin_positions = (torch.arange(-self.num_bins / 2, self.num_bins / 2) + 0.5) * self.bin_width
        if bin_type == "symmetric":
            if self.num_bins % 2 == 0:
                self.center_offset = -torch.tensor([self.bin_width / 2], dtype=torch.float32)
            else:
                self.center_offset = torch.tensor([0], dtype=torch.float32)


def _detector_ids(tc, tsm, tm, trs, ac, asm, am, ars, info):
    ids_ring = (ac + asm * info["crystalAxialNr"]
                + am * info["crystalAxialNr"] * info["submoduleAxialNr"]
                + ars * info["crystalAxialNr"] * info["submoduleAxialNr"] * info["moduleAxialNr"])
    ids_within = (tc + tsm * info["crystalTransNr"]
                  + tm * info["crystalTransNr"] * info["submoduleTransNr"]
                  + trs * info["crystalTransNr"] * info["submoduleTransNr"] * info["moduleTransNr"])
    per_ring = (info["crystalTransNr"] * info["moduleTransNr"] * info["submoduleTransNr"]
                * info["rsectorTransNr"])
    return ids_ring * per_ring + ids_within


def get_scanner_LUT(info: dict) -> torch.Tensor:
    """[n_det, 3] crystal centres (mm), sorted by detector id."""
    ar = lambda k: torch.arange(0, info[k])  # noqa: E731
    tc, ac, tsm, asm, tm, am, trs, ars = torch.cartesian_prod(
        ar("crystalTransNr"), ar("crystalAxialNr"), ar("submoduleTransNr"),
        ar("submoduleAxialNr"), ar("moduleTransNr"), ar("moduleAxialNr"), ar("rsectorTransNr"),
        ar("rsectorAxialNr")).T
    ids = _detector_ids(tc, tsm, tm, trs, ac, asm, am, ars, info)
    zm = am * info["moduleAxialSpacing"] - (info["moduleAxialNr"] - 1) * info["moduleAxialSpacing"] / 2
    zs = zm + asm * info["submoduleAxialSpacing"] - (info["submoduleAxialNr"] - 1) * info["submoduleAxialSpacing"] / 2
    zc = zs + ac * info["crystalAxialSpacing"] - (info["crystalAxialNr"] - 1) * info["crystalAxialSpacing"] / 2
    ym = tm * info["moduleTransSpacing"] - (info["moduleTransNr"] - 1) * info["moduleTransSpacing"] / 2
    ys = ym + tsm * info["submoduleTransSpacing"] - (info["submoduleTransNr"] - 1) * info["submoduleTransSpacing"] / 2
    yc = ys + tc * info["crystalTransSpacing"] - (info["crystalTransNr"] - 1) * info["crystalTransSpacing"] / 2
    xc = info["radius"] * torch.ones(len(yc))
    ang = trs / info["rsectorTransNr"] * 2 * np.pi
    rot = torch.stack([torch.cos(ang), -torch.sin(ang), torch.sin(ang), torch.cos(ang)],
                      dim=1).view(-1, 2, 2)
    xy = torch.einsum("ijk,ki->ij", rot, torch.vstack([xc, yc]))
    if info["firstCrystalAxis"] == 0:
        xy = xy.flip(dims=(1,))
    xyz = torch.vstack([xy.T, -zc.unsqueeze(0)]).T
    return xyz[torch.argsort(ids)]


class PETLMProjMeta:
    """Listmode events (detector id pairs, optional TOF bin) and scanner LUT."""

    def __init__(self, detector_ids: torch.Tensor, info: dict | None = None,
                 scanner_LUT: torch.Tensor | None = None, tof_meta: PETTOFMeta | None = None,
                 weights: torch.Tensor | None = None,
                 detector_ids_sensitivity: torch.Tensor | None = None,
                 weights_sensitivity: torch.Tensor | None = None):
        self.shape = (detector_ids.shape[0],)
        self.info = info
        self.detector_ids = detector_ids.cpu()
        self.detector_ids_sensitivity = (None if detector_ids_sensitivity is None
                                         else detector_ids_sensitivity.cpu())
        self.scanner_lut = get_scanner_LUT(info).cpu() if scanner_LUT is None else scanner_LUT
        self.tof_meta = tof_meta
        self.weights = weights
        self.weights_sensitivity = weights_sensitivity
