"""Seeded synthetic SPECT workloads with the shapes of the benchmark configurations.

The reference's tutorial datasets are not available; these phantoms stand in for them
with the stated sizes, voxel spacing, attenuation ranges and geometry.  Units follow the
reference SPECT code: cm and cm^-1.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch


@dataclass
class SpectWorkload:
    name: str
    shape: tuple
    dr: tuple
    angles: np.ndarray
    radius: float
    activity: np.ndarray
    mu: np.ndarray
    psf: tuple | None        # (a, b) of sigma(d) = a*d + b (cm), or None
    n_iters: int
    n_subsets: int
    poisson_seed: int


def _grid(shape, dr):
    axes = [(np.arange(n) - (n - 1) / 2) * d for n, d in zip(shape, dr)]
    return np.meshgrid(*axes, indexing="ij")


def config1(seed: int = 0) -> SpectWorkload:
    """64^3 at 4.8 mm, 6 ellipsoids (activities U(1,10), background 0.5), mu 0.015/mm in a
    25 cm wide ellipse, 64 angles at 25 cm, no PSF, 4 iterations x 8 subsets."""
    shape, dr = (64, 64, 64), (0.48, 0.48, 0.48)
    X, Y, Z = _grid(shape, dr)
    body = (X / 12.5) ** 2 + (Y / 10.0) ** 2 <= 1
    f = np.where(body, 0.5, 0.0)
    g = np.random.default_rng(seed)
    for _ in range(6):
        a = g.uniform(1, 4, 3)
        c = np.array([g.uniform(-12.5 + a[0], 12.5 - a[0]) * 0.6,
                      g.uniform(-10 + a[1], 10 - a[1]) * 0.6, g.uniform(-10, 10)])
        m = ((X - c[0]) / a[0]) ** 2 + ((Y - c[1]) / a[1]) ** 2 + ((Z - c[2]) / a[2]) ** 2 <= 1
        f[m & body] = g.uniform(1, 10)
    mu = np.where(body, 0.15, 0.0)
    return SpectWorkload("spect_64x64x64_64ang_att", shape, dr,
                         np.linspace(0, 360, 65)[:-1], 25.0, f, mu, None, 4, 8, 1)


def config2(seed: int = 0, n: int = 128, n_angles: int = 120) -> SpectWorkload:
    """128^3 at 4.42 mm, 3 hot spheres (8:1) in an 18x14 cm body, mu 0-0.02/mm with lung
    ellipses at 0.004/mm and a spine at 0.02/mm, 120 angles at 22 cm, PSF
    sigma(d) = 0.03 d + 0.11 cm, 4 iterations x 10 subsets."""
    shape, dr = (n, n, n), (0.442, 0.442, 0.442)
    X, Y, Z = _grid(shape, dr)
    scale = n / 128
    bx, by = 18.0 * scale, 14.0 * scale
    body = (X / bx) ** 2 + (Y / by) ** 2 <= 1
    f = np.where(body, 1.0, 0.0)
    g = np.random.default_rng(seed)
    for _ in range(3):
        r = g.uniform(1.0, 2.5) * scale
        c = np.array([g.uniform(-0.5, 0.5) * bx, g.uniform(-0.5, 0.5) * by,
                      g.uniform(-0.5, 0.5) * n * dr[2] * 0.8])
        m = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r
        f[m & body] = 8.0
    mu = np.where(body, 0.15, 0.0)
    for sx in (-1, 1):
        lung = ((X - sx * 0.45 * bx) / (0.3 * bx)) ** 2 + ((Y + 0.05 * by) / (0.55 * by)) ** 2 <= 1
        mu = np.where(lung & body, 0.04, mu)
    spine = ((X) / (0.12 * bx)) ** 2 + ((Y - 0.6 * by) / (0.12 * by)) ** 2 <= 1
    mu = np.where(spine & body, 0.2, mu)
    return SpectWorkload(f"spect_{n}x{n}x{n}_{n_angles}ang_att_psf", shape, dr,
                         np.linspace(0, 360, n_angles + 1)[:-1], 22.0, f, mu, (0.03, 0.11), 4,
                         10, 2)


def build_system_matrix(w: SpectWorkload, psf_trunc_rel: float = 1e-7):
    from .metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from .projectors.SPECT import SPECTSystemMatrix
    from .transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    om = SPECTObjectMeta(list(w.dr), w.shape)
    pm = SPECTProjMeta(w.shape[1:], list(w.dr[:2]), [float(a) for a in w.angles],
                       radii=[w.radius] * len(w.angles))
    ts = [SPECTAttenuationTransform(torch.as_tensor(w.mu, dtype=torch.float32))]
    if w.psf is not None:
        ts.append(SPECTPSFTransform(SPECTPSFMeta(w.psf)))
    return SPECTSystemMatrix(ts, [], om, pm, psf_trunc_rel=psf_trunc_rel)


def poisson_projections(H, w: SpectWorkload) -> torch.Tensor:
    """g = Poisson(H f_true), sampled on the CPU with a seeded generator."""
    f = torch.tensor(w.activity, dtype=torch.float32, device=H.device)
    clean = H.forward(f).cpu()
    gen = torch.Generator().manual_seed(w.poisson_seed)
    return torch.poisson(clean, generator=gen)


def config5(seed: int = 5, n_recons: int = 32, sizes=(64, 96, 128), angle_counts=(60, 90, 120)):
    """Uneven serving mix: n_recons seeded reconstructions with object sizes drawn from
    ``sizes`` and angle counts from ``angle_counts``, 4.42 mm voxels, 22 cm radius,
    attenuation + PSF as in the 128^3 workload (bodies scaled to the object), 10 subsets."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_recons):
        n = int(rng.choice(sizes))
        a = int(rng.choice(angle_counts))
        w = config2(seed=seed * 1000 + i, n=n, n_angles=a)
        w.poisson_seed = seed * 1000 + i
        out.append(w)
    return out
