"""Mirror of the geometry and binning helpers of src/pytomography/io/PET/shared.py.

``get_scanner_LUT`` (:360-396), ``sinogram_coordinates`` (:7-89) and
``sinogram_to_spatial`` (:91-172) are the host restatements in
``pytomography_gb300.metadata.PET``; ``listmode_to_sinogram`` (:175-272) bins on the GPU
(``gb_pet_lm_to_sino``).
"""
from __future__ import annotations

import torch

from ... import _lib
from ...metadata.PET import PETTOFMeta, get_scanner_LUT, sinogram_coordinates, \
    sinogram_to_spatial  # noqa: F401


def listmode_to_sinogram(detector_ids: torch.Tensor, info: dict,
                         weights: torch.Tensor | None = None, normalization: bool = False,
                         tof_meta: PETTOFMeta | None = None) -> torch.Tensor:
    """Sinogram [ncpr/2, ncpr+1, n_rings^2] (x TOF bins) of listmode events (detector id
    pairs, with a TOF bin column when ``tof_meta`` is given), on the CUDA device.

    Events are ordered by decreasing within-ring crystal id (a swap mirrors the TOF bin);
    the angular / radial bin and the ring-pair plane come from ``sinogram_coordinates``;
    ``normalization`` averages the ordered and the mirrored binning (shared.py:175-222);
    the TOF variant has no normalization form (shared.py:224-272)."""
    lib = _lib.load()
    if not torch.cuda.is_available():
        raise RuntimeError("listmode_to_sinogram needs a CUDA device (no CPU path)")
    dev = torch.device("cuda", torch.cuda.current_device())
    lor, sidx = sinogram_coordinates(info)
    ncpr = int(info["NrCrystalsPerRing"])
    nr = int(sidx.shape[0])
    A, R = int(ncpr / 2), ncpr + 1
    P = int((info["moduleAxialNr"] * info["crystalAxialNr"]) ** 2)
    nb = int(tof_meta.num_bins) if tof_meta is not None else 0
    ncol = 3 if nb else 2
    ev = detector_ids[:, :ncol].to(dev, torch.int32).contiguous()
    w = None if weights is None else weights.to(dev, torch.float32).contiguous()
    lor_d = lor.to(dev, torch.int32).contiguous()
    sidx_d = sidx.to(dev, torch.int32).contiguous()
    out = torch.empty((A, R, P, nb) if nb else (A, R, P), device=dev)
    _lib.check(lib.gb_pet_lm_to_sino(_lib.ptr(ev), int(ev.shape[0]), ncol, _lib.ptr(w),
                                     _lib.ptr(lor_d), _lib.ptr(sidx_d), ncpr, nr, A, R, P, nb,
                                     1 if (normalization and not nb) else 0, _lib.ptr(out),
                                     _lib.stream_handle(dev)))
    return out
