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


# ------------------------------------------------------------------- PET listmode
PET_INFO = dict(crystalTransNr=1, crystalTransSpacing=4.0, submoduleTransNr=1,
                submoduleTransSpacing=0.0, moduleTransNr=1, moduleTransSpacing=0.0,
                rsectorTransNr=600, crystalAxialNr=96, crystalAxialSpacing=4.0,
                submoduleAxialNr=1, submoduleAxialSpacing=0.0, moduleAxialNr=1,
                moduleAxialSpacing=0.0, rsectorAxialNr=1, radius=400.0, firstCrystalAxis=1,
                NrCrystalsPerRing=600, NrRings=96)


@dataclass
class PetWorkload:
    name: str
    shape: tuple
    voxel_mm: tuple
    info: dict
    events: np.ndarray      # [E, 3] int64: crystal id 1, crystal id 2, TOF bin
    tof: tuple              # (num_bins, tof_range_mm, fwhm_mm)
    randoms_per_bin: float  # additive term per event (expected randoms per LOR and TOF bin)
    n_iters: int
    n_subsets: int


def config3(seed: int = 3, n_events: int = 10_000_000, randoms_fraction: float = 0.2,
            info: dict | None = None, shape=(200, 200, 96), voxel_mm=(2.0, 2.0, 2.0),
            tof=(13, 650.0, 58.5)) -> PetWorkload:
    """TOF listmode events of an ellipsoid phantom (semi-axes 150 x 100 x 80 mm with two
    4:1 hot spheres) on a 600-crystal x 96-ring scanner of radius 400 mm: true events are
    emission points drawn from the phantom with isotropic directions that hit the
    scanner, their TOF bin drawn from the Gaussian TOF kernel around the emission point;
    randoms are uniform crystal pairs with uniform TOF bins."""
    info = dict(PET_INFO if info is None else info)
    rng = np.random.default_rng(seed)
    n_rand = int(n_events * randoms_fraction)
    n_true = n_events - n_rand
    R = info["radius"]
    n_tr = info["NrCrystalsPerRing"]
    n_ring = info["NrRings"]
    dz = info["crystalAxialSpacing"]
    z_half = (n_ring - 1) * dz / 2
    nb, tof_range, fwhm = tof
    bw = tof_range / nb
    sig = fwhm / 2.355
    chunks = []
    got = 0
    while got < n_true:
        m = 2 * (n_true - got) + 1000
        # emission points: ellipsoid with two hot spheres (rejection sampling by activity)
        p = rng.uniform(-1, 1, (m, 3)) * np.array([150.0, 100.0, 80.0])
        inside = (p[:, 0] / 150) ** 2 + (p[:, 1] / 100) ** 2 + (p[:, 2] / 80) ** 2 <= 1
        hot = ((p[:, 0] - 50) ** 2 + p[:, 1] ** 2 + p[:, 2] ** 2 <= 25.0 ** 2) | \
              ((p[:, 0] + 60) ** 2 + (p[:, 1] - 30) ** 2 + (p[:, 2] - 20) ** 2 <= 15.0 ** 2)
        act = np.where(hot, 4.0, 1.0) * inside
        keep = rng.uniform(0, 4.0, m) < act
        p = p[keep]
        u = rng.normal(size=(len(p), 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        # intersections with the cylinder x^2 + y^2 = R^2
        a = u[:, 0] ** 2 + u[:, 1] ** 2
        b = 2 * (p[:, 0] * u[:, 0] + p[:, 1] * u[:, 1])
        c = p[:, 0] ** 2 + p[:, 1] ** 2 - R ** 2
        disc = np.sqrt(np.maximum(b * b - 4 * a * c, 0))
        t1 = (-b - disc) / (2 * a + 1e-30)
        t2 = (-b + disc) / (2 * a + 1e-30)
        q1 = p + t1[:, None] * u
        q2 = p + t2[:, None] * u
        ok = (np.abs(q1[:, 2]) <= z_half) & (np.abs(q2[:, 2]) <= z_half) & (a > 1e-6)
        p, q1, q2 = p[ok], q1[ok], q2[ok]

        def crystal(q):
            phi = np.arctan2(q[:, 1], q[:, 0]) % (2 * np.pi)
            tr = np.rint(phi / (2 * np.pi / n_tr)).astype(np.int64) % n_tr
            ring = np.clip(np.rint((z_half - q[:, 2]) / dz).astype(np.int64), 0, n_ring - 1)
            return ring * n_tr + tr

        i1, i2 = crystal(q1), crystal(q2)
        # TOF: signed distance of the emission point from the LOR centre towards crystal 2
        mid = (q1 + q2) / 2
        d = q2 - q1
        s = np.einsum("ij,ij->i", p - mid, d / np.linalg.norm(d, axis=1, keepdims=True))
        s += rng.normal(0, sig, len(s))
        tb = np.clip(np.rint(s / bw).astype(np.int64) + (nb - 1) // 2, 0, nb - 1)
        good = i1 != i2
        chunks.append(np.stack([i1[good], i2[good], tb[good]], 1))
        got += int(good.sum())
    trues = np.concatenate(chunks)[:n_true]
    ri = rng.integers(0, n_tr * n_ring, n_rand)
    rj = rng.integers(0, n_tr * n_ring - 1, n_rand)
    rj = rj + (rj >= ri)
    rt = rng.integers(0, nb, n_rand)
    randoms = np.stack([ri, rj, rt], 1)
    ev = np.concatenate([trues, randoms])
    ev = ev[rng.permutation(len(ev))]
    n_det = n_tr * n_ring
    per_bin = n_rand / (n_det * (n_det - 1) / 2 * nb)
    return PetWorkload(f"pet_lm_tof_{shape[0]}x{shape[1]}x{shape[2]}_{n_events // 1_000_000}M",
                       shape, voxel_mm, info, ev, tof, per_bin, 2, 20)


def build_pet_system_matrix(w: PetWorkload, compute_sensitivity: bool = False):
    from .metadata import ObjectMeta
    from .metadata.PET import PETLMProjMeta, PETTOFMeta
    from .projectors.PET import PETLMSystemMatrix
    nb, rng_mm, fwhm = w.tof
    pm = PETLMProjMeta(torch.as_tensor(w.events), info=w.info,
                       tof_meta=PETTOFMeta(nb, rng_mm, fwhm))
    return PETLMSystemMatrix(ObjectMeta(list(w.voxel_mm), w.shape), pm,
                             compute_sensitivity=compute_sensitivity)
