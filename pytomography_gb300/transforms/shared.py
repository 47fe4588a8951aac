"""Object-space plugins either side of the projectors.

* ``GaussianFilter`` (src/pytomography/transforms/shared/filters.py:8-80): separable
  Gaussian smoothing with per-axis kernels of ``2 ceil(n_sigmas sigma / dr) + 1`` taps,
  ``exp(-x^2 / (2 sigma^2))`` normalised, 'same' zero padding, x then y then z; the
  operator is symmetric, so ``backward`` is ``forward``.  Used as the resolution model of
  the PET system matrices (applied before forward projection and after back projection).
* ``KEMTransform`` (src/pytomography/transforms/shared/kem.py:10-138): the kernel-method
  basis f = K alpha.  ``compute_kernel`` follows the reference's construction (product of
  support kernels of each support object against its replicate-padded neighbour, optional
  top-N selection per voxel, distance kernel, normalisation over the neighbourhood);
  the table is kept on the GPU and applied by ``gb_kem_apply``.  ``backward`` is
  ``forward``, as in the reference.

Both apply through CUDA kernels of ``libgbtomo.so``; there is no CPU path.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _lib
from .transform import Transform


def _device_of(t: torch.Tensor | None = None):
    if not torch.cuda.is_available():
        raise RuntimeError("object-space transforms need a CUDA device (no CPU path)")
    if t is not None and t.is_cuda:
        return t.device
    return torch.device("cuda", torch.cuda.current_device())


class GaussianFilter(Transform):
    """Gaussian smoothing with the given FWHM (units of the object's voxel size)."""

    def __init__(self, FWHM: float, n_sigmas: float = 3):
        super().__init__()
        self.sigma = FWHM / (2 * np.sqrt(2 * np.log(2)))
        self.n_sigmas = n_sigmas

    def configure(self, object_meta, proj_meta) -> None:
        self.object_meta = object_meta
        self.proj_meta = proj_meta
        self._get_kernels()

    def _get_kernels(self) -> None:
        self.kernels = []
        for i in range(3):
            dx = self.object_meta.dr[i]
            size = int(2 * np.ceil(self.n_sigmas * self.sigma / dx) + 1)
            x = torch.arange(-int(size // 2), int(size // 2) + 1) * dx
            k = torch.exp(-x ** 2 / (2 * self.sigma ** 2))
            self.kernels.append((k / k.sum()).to(torch.float32))
        self._taps_dev = None

    def __call__(self, object):
        return self.forward(object)

    def forward(self, object: torch.Tensor) -> torch.Tensor:
        dev = _device_of(object)
        if self._taps_dev is None or self._taps_dev[0].device != dev:
            self._taps_dev = [k.to(dev).contiguous() for k in self.kernels]
        x = object.to(dev, torch.float32).contiguous()
        out = torch.empty_like(x)
        scratch = torch.empty_like(x)
        nx, ny, nz = (int(s) for s in x.shape)
        tx, ty, tz = self._taps_dev
        lib = _lib.load()
        _lib.check(lib.gb_filter3d(_lib.ptr(x), _lib.ptr(out), _lib.ptr(scratch), nx, ny, nz,
                                   _lib.ptr(tx), tx.numel(), _lib.ptr(ty), ty.numel(),
                                   _lib.ptr(tz), tz.numel(), _lib.stream_handle(dev)))
        return out

    def backward(self, object, norm_constant=None):
        object = self.forward(object)
        if norm_constant is not None:
            return object, self.forward(norm_constant)
        return object


def _neighbour(obj: torch.Tensor, shift) -> torch.Tensor:
    """obj[clamp(x + i), clamp(y + j), clamp(z + k)] (get_object_nearest_neighbour,
    utils/misc.py:40-57)."""
    i, j, k = (int(s) for s in shift)
    nx, ny, nz = obj.shape
    ix = torch.clamp(torch.arange(nx) + i, 0, nx - 1)
    iy = torch.clamp(torch.arange(ny) + j, 0, ny - 1)
    iz = torch.clamp(torch.arange(nz) + k, 0, nz - 1)
    return obj[ix][:, iy][:, :, iz]


class KEMTransform(Transform):
    """Kernel-method basis K; ``forward(alpha) = K alpha``."""

    def __init__(self, support_objects, support_kernels=None, support_kernels_params=None,
                 distance_kernel=None, distance_kernel_params=None, size: int = 5,
                 top_N: int | None = None, kernel_on_gpu: bool = True) -> None:
        super().__init__()
        self.support_objects = support_objects
        if support_kernels is None:
            self.support_kernels = [
                lambda a, b, sigma: torch.exp(-(a - b) ** 2 / (2 * sigma ** 2))
                for _ in range(len(support_objects))]
        else:
            self.support_kernels = support_kernels
        self.support_kernel_params = ([[1] for _ in range(len(support_objects))]
                                      if support_kernels_params is None
                                      else support_kernels_params)
        self.distance_kernel = (distance_kernel if distance_kernel is not None
                                else lambda d, sigma: torch.exp(-d ** 2 / (2 * sigma ** 2)))
        self.distance_kernel_params = [1] if distance_kernel_params is None \
            else distance_kernel_params
        self.size = size
        self.idx_max = int((size - 1) / 2)
        self.idxs = torch.arange(-self.idx_max, self.idx_max + 1)
        self.top_N = top_N
        self.kernel_on_gpu = kernel_on_gpu

    def compute_kernel(self) -> None:
        """[size^3][shape] weights (kem.py:69-95), built on the CPU like the reference (the
        top-N ranking breaks ties the same way), then kept on the GPU."""
        shape = tuple(self.support_objects[0].shape)
        s = self.size
        kern = torch.ones((s, s, s, *shape), dtype=torch.float32)
        sup = [o.detach().to("cpu", torch.float32) for o in self.support_objects]
        for i in self.idxs:
            for j in self.idxs:
                for k in self.idxs:
                    comp = 1
                    for lidx, o in enumerate(sup):
                        comp = comp * self.support_kernels[lidx](
                            o, _neighbour(o, (i, j, k)), *self.support_kernel_params[lidx])
                    kern[i + self.idx_max, j + self.idx_max, k + self.idx_max] = comp
        if self.top_N is not None:
            flat = kern.reshape((s ** 3, *shape))
            rank = torch.argsort(torch.argsort(flat, dim=0), dim=0)
            kern *= (rank >= s ** 3 - self.top_N).reshape((s, s, s, *shape))
        om = self.object_meta
        xv, yv, zv = torch.meshgrid([om.dx * self.idxs, om.dy * self.idxs, om.dz * self.idxs],
                                    indexing="ij")
        d = torch.sqrt(xv ** 2 + yv ** 2 + zv ** 2)
        dk = torch.as_tensor(self.distance_kernel(d, *self.distance_kernel_params),
                             dtype=torch.float32)
        kern *= dk.reshape(s, s, s, *([1] * len(shape)))
        kern /= kern.sum(dim=(0, 1, 2))
        self.kernel = kern
        self._kern_dev = kern.reshape(s ** 3, *shape).to(_device_of()).contiguous()

    def configure(self, object_meta, proj_meta) -> None:
        super().configure(object_meta, proj_meta)
        self.compute_kernel()

    @torch.no_grad()
    def forward(self, object: torch.Tensor) -> torch.Tensor:
        dev = self._kern_dev.device
        x = object.to(dev, torch.float32).contiguous()
        out = torch.empty_like(x)
        nx, ny, nz = (int(v) for v in x.shape)
        _lib.check(_lib.load().gb_kem_apply(_lib.ptr(x), _lib.ptr(out), _lib.ptr(self._kern_dev),
                                            nx, ny, nz, int(self.size),
                                            _lib.stream_handle(dev)))
        return out

    @torch.no_grad()
    def backward(self, object: torch.Tensor) -> torch.Tensor:
        return self.forward(object)
