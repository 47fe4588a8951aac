"""Host-side geometry tables of the SPECT projector.

* pad sizes (``compute_pad_size`` / ``compute_pad_size_padded``,
  src/pytomography/utils/spatial.py:36-62);
* detector distances per plane (``get_distance``, src/pytomography/utils/misc.py:21-38);
* the normalised sampling matrix of a kornia-convention rotation.  kornia is a
  third-party dependency of the reference (``kornia>=0.6.12``, pyproject.toml:25) used at
  src/pytomography/utils/spatial.py:31,33 and transforms/shared/spatial.py:36,53.  Its
  published algorithm builds ``M = T(c) R(angle) T(-c)`` with
  ``R = [[cos, sin], [-sin, cos]]`` about ``c = ((W-1)/2, (H-1)/2)``, conjugates it into
  normalised coordinates ``N = [[2/(W-1), 0, -1], [0, 2/(H-1), -1], [0, 0, 1]]`` and
  samples with the inverse (``affine_grid`` / ``grid_sample``, bilinear, zeros,
  ``align_corners=True``).  The matrices are computed here in float32 with the same
  operation sequence, so the CUDA kernels sample at the reference's coordinates;
* per-plane PSF taps (``SPECTPSFTransform._get_sigma/_compute_kernel_size`` and
  ``get_1D_PSF_layer_gaussian/_square``, src/pytomography/transforms/SPECT/psf.py:62-99,
  170-197), computed in float32 torch on the CPU like the reference's Conv1d weights.
"""
from __future__ import annotations

import math

import numpy as np
import torch

DELTA = 1e-11


def compute_pad_size(width: int) -> int:
    return int(np.ceil((np.sqrt(2) * width - width) / 2))


def compute_pad_size_padded(width: int) -> int:
    a = (np.sqrt(2) - 1) / 2
    if width % 2 == 0:
        width_old = int(2 * np.floor((width / 2) / (1 + 2 * a)))
    else:
        width_old = int(2 * np.floor(((width - 1) / 2) / (1 + 2 * a)))
    return int((width - width_old) / 2)


def get_distance(Lx: int, r: float, dx: float) -> np.ndarray:
    if Lx % 2 == 0:
        d = r + (Lx / 2 - np.arange(Lx) - 1 / 2) * dx
    else:
        d = r + ((Lx - 1) / 2 - np.arange(Lx)) * dx
    d[d < 0] = 0
    return d


def rotation_theta(angle_deg: torch.Tensor, size: int) -> torch.Tensor:
    """[n, 6] float32 sampling matrices (dst -> src, normalised) for rotations of a
    ``size`` x ``size`` image by ``angle_deg`` (counter-clockwise positive)."""
    dt = torch.float32
    angle = torch.as_tensor(angle_deg, dtype=dt).reshape(-1).cpu()
    B = angle.shape[0]
    c = (size - 1) / 2.0
    center = torch.tensor([c, c], dtype=dt).expand(B, 2)
    pi = torch.tensor(math.pi, dtype=dt)
    ang = angle * pi / 180.0
    cs, sn = torch.cos(ang), torch.sin(ang)
    rot = torch.stack([cs, sn, -sn, cs], dim=-1).view(B, 2, 2)
    eye = torch.eye(3, dtype=dt).expand(B, 3, 3)
    t_pos = eye.clone()
    t_pos[:, :2, 2] = center
    t_neg = eye.clone()
    t_neg[:, :2, 2] = -center
    r3 = eye.clone()
    r3[:, :2, :2] = rot
    pix = t_pos @ r3 @ eye.clone() @ t_neg
    pix3 = eye.clone()
    pix3[:, :2, :] = pix[:, :2, :]
    nrm = torch.tensor([[1.0, 0.0, -1.0], [0.0, 1.0, -1.0], [0.0, 0.0, 1.0]], dtype=dt)
    nrm[0, 0] = nrm[0, 0] * 2.0 / (size - 1.0)
    nrm[1, 1] = nrm[1, 1] * 2.0 / (size - 1.0)
    nrm = nrm.unsqueeze(0)
    fwd_norm = nrm @ (pix3 @ torch.inverse(nrm))
    theta = torch.inverse(fwd_norm)[:, :2, :]
    return theta.reshape(B, 6).contiguous()


def base_grid(size: int) -> torch.Tensor:
    """Normalised pixel-centre coordinates used by ``affine_grid(align_corners=True)``."""
    return torch.linspace(-1, 1, size, dtype=torch.float32)


def psf_sigma(n_pad: int, radius: float, dx: float, psf_meta) -> np.ndarray:
    distances = get_distance(n_pad, radius, dx)
    return psf_meta.sigma_fit(distances, *psf_meta.sigma_fit_params)


def psf_kernel_size(sigma: np.ndarray, dr_axis: float, min_sigmas: float) -> int:
    sigma_max = max(sigma) / dr_axis
    return int((np.ceil(sigma_max * min_sigmas) * 2 + 1).astype(int))


def psf_taps(sigmas_px: np.ndarray, kernel_size: int, shape: str = "gaussian") -> torch.Tensor:
    """[len(sigmas), kernel_size] float32 taps, normalised per plane."""
    N = len(sigmas_px)
    x = torch.arange(-int(kernel_size // 2), int(kernel_size // 2) + 1).unsqueeze(0).unsqueeze(0)
    x = x.repeat((N, 1, 1))
    sig = torch.tensor(sigmas_px).to(torch.float32).reshape((N, 1, 1))
    if shape == "gaussian":
        k = torch.exp(-x ** 2 / (2 * sig ** 2 + DELTA))
    elif shape == "square":
        k = 1 - torch.abs(x) / sig
        k[k < 0] = 0
    else:
        raise NotImplementedError(f"PSF shape {shape!r}")
    k = k / k.sum(axis=-1).unsqueeze(-1)
    return k.to(torch.float32)[:, 0, :]
