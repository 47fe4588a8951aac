"""PET metadata mirrors.

``PETTOFMeta`` (src/pytomography/metadata/PET/pet_tof_metadata.py:5-37),
``PETLMProjMeta`` (src/pytomography/metadata/PET/petlm_metadata.py:6-39),
``PETSinogramPolygonProjMeta`` (src/pytomography/metadata/PET/pet_sinogram_metadata.py:
6-26), the scanner lookup table builder ``get_scanner_LUT`` and the sinogram geometry
tables ``sinogram_coordinates`` / ``sinogram_to_spatial``
(src/pytomography/io/PET/shared.py:7-172, 275-396).
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


# ---------------------------------------------------------------- sinograms
def _lor_bins(ncpr: int, d0: float, min_diff: int, radial_size: int):
    """(angular, radial) sinogram bin of every ordered pair of within-ring crystal ids,
    with the validity mask (shared.py:22-63): crystal ids are counted from the centre of
    the first sector, a pair's radial offset and angle follow from the smaller and larger
    id and their sum."""
    c = np.arange(ncpr, dtype=np.float64) - d0
    c = np.where(c < 0, c + ncpr, c)
    c1, c2 = np.meshgrid(c, c, indexing="ij")
    a, b = np.minimum(c1, c2), np.maximum(c1, c2)
    valid = (b - a) >= min_diff
    s = a + b
    outer = (s >= 1.5 * ncpr) | (s < 0.5 * ncpr)
    span = (b - a - 1) / 2 - (ncpr - (b - a + 1)) / 2
    radial = np.where(outer, np.where(a == b, -ncpr / 2, span),
                      np.where(a == b, ncpr / 2, -span))
    radial = np.floor(radial)
    angular = np.where(s < ncpr / 2, (2 * a + ncpr + radial) / 2,
                       np.where(s >= 1.5 * ncpr, (2 * a - ncpr + radial) / 2,
                                (2 * a - radial) / 2))
    return np.floor(angular), np.floor(radial + radial_size / 2), valid


def _ring_pair_index(nr: int) -> np.ndarray:
    """[nr, nr] sinogram plane of each ring pair (shared.py:64-83): ring differences in
    increasing order, both orders of a pair in consecutive blocks."""
    r1, r2 = np.meshgrid(np.arange(1, nr + 1), np.arange(1, nr + 1), indexing="ij")
    rd = np.abs(r2 - r1)
    before = nr + 2 * (rd - 1) * nr - (rd - 1) * rd  # planes of smaller differences
    idx = np.where(rd == 0, r1, np.where(r1 < r2, before + r1, before + nr - rd + r1 - rd))
    return idx - 1


def sinogram_coordinates(info: dict):
    """[ncpr, ncpr, 2] (angular, radial) bin of each crystal pair and [nr, nr] sinogram
    plane of each ring pair (shared.py:7-89)."""
    ncpr, nr = int(info["NrCrystalsPerRing"]), int(info["NrRings"])
    min_diff = info["min_rsector_difference"] * info["moduleTransNr"] * info["crystalTransNr"]
    radial_size = ncpr - 2 * (min_diff - 1) - 1
    d0 = info["moduleTransNr"] * info["crystalTransNr"] / 2
    ang, rad, valid = _lor_bins(ncpr, d0, min_diff, radial_size)
    lor = np.zeros((ncpr, ncpr, 2), np.int64)
    lor[..., 0] = np.where(valid, ang, 0)
    lor[..., 1] = np.where(valid, rad, 0)
    return torch.tensor(lor), torch.tensor(_ring_pair_index(nr), dtype=torch.long)


def sinogram_to_spatial(info: dict):
    """[ncpr/2, ncpr+1, 2, 2] transaxial (x, y) of the two crystals of every sinogram bin
    and [nr*nr, 2] axial z of the two rings of every sinogram plane (shared.py:91-172).
    A bin reached by several crystal pairs keeps the last pair in (crystal 1, crystal 2)
    loop order; bins no pair reaches stay at (0, 0)."""
    lut = get_scanner_LUT(info).numpy()
    nr = info["rsectorAxialNr"] * info["moduleAxialNr"] * info["crystalAxialNr"]
    ncpr = info["rsectorTransNr"] * info["moduleTransNr"] * info["crystalTransNr"]
    radial_size, angular_size = int(ncpr + 1), int(ncpr / 2)
    d0 = info["moduleTransNr"] * info["crystalTransNr"] / 2
    ang, rad, _ = _lor_bins(ncpr, d0, 0, radial_size)
    c1, c2 = np.meshgrid(np.arange(ncpr), np.arange(ncpr), indexing="ij")
    keep = (c1 >= c2).ravel()
    ai, ri = ang.ravel().astype(np.int64)[keep], rad.ravel().astype(np.int64)[keep]
    k1, k2 = c1.ravel()[keep], c2.ravel()[keep]
    det = np.zeros((angular_size, radial_size, 2, 2), np.float32)
    # last write wins: keep the final occurrence of every target bin in loop order
    flat = ai * radial_size + ri
    rev_first = np.unique(flat[::-1], return_index=True)[1]
    last = len(flat) - 1 - rev_first
    det[ai[last], ri[last], 0, :] = lut[k1[last], 0:2]
    det[ai[last], ri[last], 1, :] = lut[k2[last], 0:2]
    pidx = _ring_pair_index(nr)
    ring = np.zeros((nr * nr, 2), np.float32)
    r1, r2 = np.meshgrid(np.arange(nr), np.arange(nr), indexing="ij")
    ring[pidx.ravel(), 0] = lut[info["NrCrystalsPerRing"] * r1.ravel(), 2]
    ring[pidx.ravel(), 1] = lut[info["NrCrystalsPerRing"] * r2.ravel(), 2]
    return torch.tensor(det), torch.tensor(ring)


class PETSinogramPolygonProjMeta:
    """Sinogram [n_angles, n_radial, n_planes] (x TOF bins) of a polygonal scanner."""

    def __init__(self, info: dict, tof_meta: PETTOFMeta | None = None):
        self.info = info
        self.scanner_lut = get_scanner_LUT(info)
        self.detector_coordinates, self.ring_coordinates = sinogram_to_spatial(info)
        self.shape = [self.detector_coordinates.shape[0], self.detector_coordinates.shape[1],
                      self.ring_coordinates.shape[0]]
        self.N_angles = self.detector_coordinates.shape[0]
        self.tof_meta = tof_meta
