"""Multi-bed SPECT stitching (mirror of ``stitch_multibed``, src/pytomography/io/SPECT/
dicom.py:599-653) with the bed positions given directly instead of read from DICOM
headers (DICOM IO is not part of this package).

Beds are ordered by increasing z; bed i starts at slice round((z_i - z_0) / spacing) of the
stitched volume.  Each bed's first and last slice are dropped, and an overlap with the
next bed is split at its middle: the lower bed keeps the lower half, the upper bed the
upper half (the reference's mid-slice stitch).
"""
from __future__ import annotations

from collections.abc import Sequence

import numpy as np
import torch


def stitching_layout(bed_z: Sequence[float], slice_spacing: float, n_slices: int):
    """(order, start slice per sorted bed, z weight profile [n_beds, n_slices] per sorted
    bed) of the mid-slice stitch."""
    z = np.asarray(bed_z, dtype=np.float64)
    order = np.argsort(z)
    zs = np.round((z[order] - z[order][0]) / slice_spacing).astype(int)
    below, above = 1, n_slices - 1
    w = np.zeros((len(z), n_slices), np.float32)
    w[:, below:above] = 1
    for i in range(len(z) - 1):
        lower = zs[i + 1] - zs[i] + below
        delta = above - lower
        half = round(delta / 2)
        w[i, lower + half:lower + delta] = 0
        w[i + 1, below:below + half] = 0
    return order, zs, w


def stitch_multibed(recons: torch.Tensor, bed_z: Sequence[float], slice_spacing: float,
                    return_stitching_weights: bool = False):
    """Stitch reconstructions [n_beds, Lx, Ly, Lz] of beds at z positions ``bed_z`` (same
    units as ``slice_spacing``) into [Lx, Ly, Lz'].  With ``return_stitching_weights`` it
    returns each bed's weights [n_beds, Lx, Ly, Lz] and start slice, in the input order."""
    n, lx, ly, lz = recons.shape
    order, zs, w = stitching_layout(bed_z, slice_spacing, lz)
    wt = torch.tensor(w, device=recons.device)
    if return_stitching_weights:
        inv = np.argsort(order)
        weights = wt[torch.as_tensor(inv)].view(n, 1, 1, lz).expand(n, lx, ly, lz).clone()
        return weights, zs[inv]
    out = torch.zeros((lx, ly, int(zs[-1]) + lz), device=recons.device, dtype=recons.dtype)
    for i, b in enumerate(order):
        out[:, :, zs[i]:zs[i] + lz] += recons[int(b)] * wt[i]
    return out
