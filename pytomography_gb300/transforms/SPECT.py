"""SPECT obj2obj plugins: attenuation and depth-dependent Gaussian PSF.

Mirrors of ``SPECTAttenuationTransform`` (src/pytomography/transforms/SPECT/attenuation.py:24-115)
and ``SPECTPSFTransform`` (src/pytomography/transforms/SPECT/psf.py:101-231).

Two uses:

* inside this package's ``SPECTSystemMatrix`` the plugins are lowered into the fused CUDA
  plan (the attenuation factor and the per-plane blur run inside the projector kernels);
* called on their own, ``forward(object_i, ang_idx)`` / ``backward(object_i, ang_idx)``
  act on an object already padded and rotated into the detector frame of projection
  ``ang_idx``, as in the reference's per-angle loop
  (projectors/SPECT/spect_system_matrix.py:145-154, 188-198).  Each call is one CUDA
  kernel (``gb_spect_attenuation_apply`` / ``gb_spect_psf_apply``); the object must be a
  CUDA float32 tensor, there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib, geometry
from .transform import Transform


def _angle_index(ang_idx) -> int:
    if isinstance(ang_idx, torch.Tensor):
        if ang_idx.numel() != 1:
            raise NotImplementedError("one projection index per plugin call")
        return int(ang_idx.reshape(-1)[0].item())
    return int(ang_idx)


def _object_in(x: torch.Tensor, shape, name: str) -> torch.Tensor:
    if tuple(x.shape) != tuple(shape):
        raise ValueError(f"{name}: expected an object of shape {tuple(shape)}, got {tuple(x.shape)}")
    if not x.is_cuda:
        raise RuntimeError(f"{name}: the plugin runs on the GPU only (no CPU path)")
    return x.to(torch.float32).contiguous()


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
        self._dev = None

    def configure(self, object_meta, proj_meta) -> None:
        super().configure(object_meta, proj_meta)
        n = int(object_meta.shape[0])
        self._pad = geometry.compute_pad_size(n) if self.assume_padded else 0
        self._L = n + 2 * self._pad
        self._theta_cache = None  # built on the first per-angle call (fused plans skip it)
        self._dev = None

    @property
    def _theta(self) -> np.ndarray:
        if self._theta_cache is None:
            angles = torch.as_tensor(self.proj_meta.angles, dtype=torch.float32).reshape(-1).cpu()
            # the map is sampled with the forward projector's rotation, angle beta - 270
            # (utils/spatial.py:29-31 through rotate_detector_z)
            self._theta_cache = geometry.rotation_theta(-(270 - angles), self._L).numpy()
        return self._theta_cache

    def _device_tables(self, device):
        if self._dev is None or self._dev[0] != device:
            mu = self.attenuation_map.to(device, torch.float32).contiguous()
            lin = geometry.base_grid(self._L).to(device)
            self._dev = (device, mu, lin)
        return self._dev[1], self._dev[2]

    def _apply(self, object_i: torch.Tensor, ang_idx) -> torch.Tensor:
        lib = _lib.load()
        n, _, nz = (int(s) for s in self.object_meta.shape)
        x = _object_in(object_i, (self._L, self._L, nz), "SPECTAttenuationTransform")
        mu, lin = self._device_tables(x.device)
        th = np.ascontiguousarray(self._theta[_angle_index(ang_idx)], dtype=np.float32)
        out = torch.empty_like(x)
        with torch.cuda.device(x.device):
            _lib.check(lib.gb_spect_attenuation_apply(
                _lib.ptr(mu), n, nz, self._pad, float(self.object_meta.dx),
                th.ctypes.data_as(ctypes.c_void_p), _lib.ptr(lin), _lib.ptr(x), _lib.ptr(out),
                _lib.stream_handle(x.device)))
        return out

    def forward(self, object_i: torch.Tensor, ang_idx) -> torch.Tensor:
        """object_i [L, L, Lz] in the detector frame of projection ``ang_idx`` times the
        probability of detection at +x (attenuation.py:72-92)."""
        return self._apply(object_i, ang_idx)

    def backward(self, object_i: torch.Tensor, ang_idx) -> torch.Tensor:
        """The same diagonal operator (attenuation.py:94-115)."""
        return self._apply(object_i, ang_idx)


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
        self._dev_tables = {}

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
            two_d = self.psf_meta.kernel_dimensions == "2D"
            if not two_d:
                wz = None
            elif kz == kr and float(self.object_meta.dz) == float(self.object_meta.dx):
                wz = wr  # cubic voxels: the same arguments give the same taps
            else:
                wz = geometry.psf_taps(sigma / self.object_meta.dz, kz, self.psf_meta.shape)
            self.tables[radius] = (wr, wz)
        self._dev_tables = {}

    def _taps_on(self, radius: float, device):
        key = (radius, str(device))
        hit = self._dev_tables.get(key)
        if hit is None:
            wr, wz = self.tables[radius]
            hit = (wr.to(device).contiguous(), None if wz is None else wz.to(device).contiguous())
            self._dev_tables[key] = hit
        return hit

    def _apply(self, object: torch.Tensor, ang_idx) -> torch.Tensor:
        lib = _lib.load()
        radius = float(self.proj_meta.radii[_angle_index(ang_idx)])
        wr, wz = self.tables[radius]
        L = int(wr.shape[0])
        _, ny, nz = (int(s) for s in object.shape)
        x = _object_in(object, (L, ny, nz), "SPECTPSFTransform")
        dwr, dwz = self._taps_on(radius, x.device)
        out = torch.empty_like(x)
        with torch.cuda.device(x.device):
            _lib.check(lib.gb_spect_psf_apply(
                _lib.ptr(x), _lib.ptr(out), L, ny, nz, _lib.ptr(dwr), int(dwr.shape[1]),
                _lib.ptr(dwz), 0 if dwz is None else int(dwz.shape[1]),
                _lib.stream_handle(x.device)))
        return out

    def forward(self, object: torch.Tensor, ang_idx) -> torch.Tensor:
        """Blur every plane x of a detector-frame object [L, Ly, Lz] with the kernel of
        its distance to the detector of projection ``ang_idx`` (psf.py:199-214)."""
        return self._apply(object, ang_idx)

    def backward(self, object: torch.Tensor, ang_idx) -> torch.Tensor:
        """The same symmetric operator (psf.py:216-231)."""
        return self._apply(object, ang_idx)
