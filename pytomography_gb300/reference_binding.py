"""The binding a PyTomography maintainer would add: the reference's own ``SPECTSystemMatrix``
driving ``libgbtomo.so`` through the C ABI.

Users who keep the reference package as their front end (its metadata, transforms,
likelihoods and algorithms) replace only the per-angle loops of
``SPECTSystemMatrix.forward`` / ``backward``
(src/pytomography/projectors/SPECT/spect_system_matrix.py:120-201):

* :func:`describe` reads a configured reference system matrix (object / projection
  metadata and its ``SPECTAttenuationTransform`` / ``SPECTPSFTransform`` plugins) into the
  fields of ``gb_spect_desc``.  The PSF taps are the reference plugin's own ``Conv1d``
  weights (transforms/SPECT/psf.py:62-83, 119-142), so the plan blurs with exactly the
  reference's kernels;
* :func:`make_plan` creates the plan (``gb_spect_plan_create``);
* :func:`bind` returns a subclass of the reference class whose ``set_n_subsets``,
  ``forward`` and ``backward`` call ``gb_spect_set_subsets`` / ``gb_spect_forward`` /
  ``gb_spect_backward`` on CUDA tensors.

Importing this module does not import the reference; :func:`bind` takes the reference
class as its argument.  Transforms other than attenuation and PSF raise
``NotImplementedError`` (there is no CPU path to fall back on).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, geometry


def _order_and_plugins(sm):
    order, mu, psf = "", None, None
    for t in sm.obj2obj_transforms:
        name = type(t).__name__
        if name == "SPECTAttenuationTransform":
            order += "a"
            mu = t.attenuation_map
        elif name == "SPECTPSFTransform":
            if getattr(t, "psf_operator", None) is not None:
                raise NotImplementedError("a psf_operator network has no fused kernel")
            order += "p"
            psf = t
        else:
            raise NotImplementedError(f"transform {name} has no fused GB300 implementation")
    if sm.proj2proj_transforms:
        raise NotImplementedError("proj2proj transforms are not part of the fused path")
    if order.count("a") > 1 or order.count("p") > 1:
        raise NotImplementedError("at most one attenuation and one PSF transform")
    return order, mu, psf


def describe(sm) -> dict:
    """The gb_spect_desc fields of a configured reference ``SPECTSystemMatrix`` (host
    arrays; ``mu`` as a float32 tensor)."""
    om, pm = sm.object_meta, sm.proj_meta
    nx, ny, nz = (int(v) for v in om.shape)
    order, mu, psf = _order_and_plugins(sm)
    pad = geometry.compute_pad_size(nx)
    Lp = nx + 2 * pad
    angles = torch.as_tensor(pm.angles, dtype=torch.float32).reshape(-1).cpu()
    d = {"nx": nx, "ny": ny, "nz": nz, "dr": tuple(float(v) for v in om.dr),
         "n_angles": int(angles.numel()), "order": order,
         # forward: RotationTransform.backward(obj, 270 - beta) = rotate(beta - 270);
         # back projection: rotate(270 - beta) (spect_system_matrix.py:150, 196)
         "theta_fwd": geometry.rotation_theta(-(270 - angles), Lp).numpy(),
         "theta_bwd": geometry.rotation_theta(270 - angles, Lp).numpy(),
         "lin": geometry.base_grid(Lp).numpy(), "pad": pad,
         "mu": None if mu is None else torch.as_tensor(mu).to(torch.float32).cpu()}
    if psf is not None:
        radii = [float(r) for r in np.unique(np.asarray(pm.radii, dtype=np.float64))]
        tabs_r, tabs_z, k, two_d = [], [], 1, True
        for r in radii:
            if hasattr(psf, "layers"):  # the reference plugin: its Conv1d layers per radius
                layer = psf.layers[r]
                wr = layer.layer_r.weight.detach().to(torch.float32).cpu().numpy()[:, 0, :]
                lz = layer.layer_z
                wz = None if not lz else lz.weight.detach().to(torch.float32).cpu().numpy()[:, 0, :]
            else:  # this package's plugin: the same taps as host tables
                wr_t, wz_t = psf.tables[r]
                wr = wr_t.numpy()
                wz = None if wz_t is None else wz_t.numpy()
            two_d = wz is not None
            tabs_r.append(wr)
            tabs_z.append(wz)
            k = max(k, wr.shape[1], 0 if wz is None else wz.shape[1])
        tr = np.zeros((len(radii), Lp, k), np.float32)
        tz = np.zeros((len(radii), Lp, k), np.float32)
        for gi, (wr, wz) in enumerate(zip(tabs_r, tabs_z)):
            o = (k - wr.shape[1]) // 2
            tr[gi, :, o:o + wr.shape[1]] = wr
            if wz is not None:
                o = (k - wz.shape[1]) // 2
                tz[gi, :, o:o + wz.shape[1]] = wz
        d.update({"psf_2d": int(two_d), "psf_k": k, "psf_taps_r": tr, "psf_taps_z": tz,
                  "psf_group": np.array([radii.index(float(r)) for r in pm.radii], np.int32),
                  "psf_radii": radii})
    return d


class Plan:
    """A ``gb_spect_plan`` with the host and device buffers its descriptor points to."""

    def __init__(self, d: dict, device, psf_trunc_rel: float = 1e-7) -> None:
        self.lib = _lib.load()
        self.desc_fields = d
        self.device = torch.device(device)
        desc = _lib.SpectDesc()
        desc.nx, desc.ny, desc.nz = d["nx"], d["ny"], d["nz"]
        desc.dx, desc.dy, desc.dz = d["dr"]
        desc.n_angles = d["n_angles"]
        self._keep = [np.ascontiguousarray(d["theta_fwd"], np.float32),
                      np.ascontiguousarray(d["theta_bwd"], np.float32),
                      np.ascontiguousarray(d["lin"], np.float32)]
        desc.theta_fwd, desc.theta_bwd, desc.lin = (a.ctypes.data_as(ctypes.c_void_p)
                                                    for a in self._keep)
        self.mu = None if d["mu"] is None else d["mu"].to(self.device).contiguous()
        desc.mu = None if self.mu is None else ctypes.c_void_p(self.mu.data_ptr())
        desc.order = d["order"].encode()
        if "psf_k" in d:
            arrs = [np.ascontiguousarray(d[k]) for k in ("psf_taps_r", "psf_taps_z", "psf_group")]
            self._keep += arrs
            desc.psf_taps_r, desc.psf_taps_z, desc.psf_group = (
                a.ctypes.data_as(ctypes.c_void_p) for a in arrs)
            desc.psf_2d, desc.psf_k = d["psf_2d"], d["psf_k"]
            desc.psf_n_groups = len(d["psf_radii"])
            desc.psf_trunc_rel = float(psf_trunc_rel)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            torch.cuda.synchronize()
            _lib.check(self.lib.gb_spect_plan_create(ctypes.byref(desc), ctypes.byref(h)))
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None:
            try:
                self.lib.gb_spect_plan_destroy(h)
            except Exception:
                pass


def make_plan(sm, device="cuda", psf_trunc_rel: float = 1e-7) -> Plan:
    """gb_spect_plan_create for a configured reference ``SPECTSystemMatrix``."""
    return Plan(describe(sm), device, psf_trunc_rel)


def bind(reference_system_matrix_class):
    """A subclass of the reference ``SPECTSystemMatrix`` whose projectors run on the GPU
    through the C ABI; constructor arguments are the reference's."""

    class GB300SPECTSystemMatrix(reference_system_matrix_class):
        def __init__(self, *args, **kwargs):
            super().__init__(*args, **kwargs)
            self._gb = make_plan(self)

        def set_n_subsets(self, n_subsets: int) -> None:
            super().set_n_subsets(n_subsets)
            _lib.check(self._gb.lib.gb_spect_set_subsets(self._gb.handle, int(n_subsets)))

        def _n_sel(self, subset_idx):
            return self.proj_meta.num_projections if subset_idx is None else \
                len(self.subset_indices_array[subset_idx])

        def forward(self, object, subset_idx=None):
            dev = self._gb.device
            obj = object.to(dev, torch.float32).contiguous()
            out = torch.empty((self._n_sel(subset_idx), *self.proj_meta.shape[1:]), device=dev)
            _lib.check(self._gb.lib.gb_spect_forward(
                self._gb.handle, _lib.ptr(obj), _lib.ptr(out),
                -1 if subset_idx is None else int(subset_idx), _lib.stream_handle(dev)))
            return out

        def backward(self, proj, subset_idx=None):
            dev = self._gb.device
            p = proj.to(dev, torch.float32).contiguous()
            out = torch.empty(tuple(self.object_meta.shape), device=dev)
            _lib.check(self._gb.lib.gb_spect_backward(
                self._gb.handle, _lib.ptr(p), _lib.ptr(out),
                -1 if subset_idx is None else int(subset_idx), 0, _lib.stream_handle(dev)))
            return out

    GB300SPECTSystemMatrix.__name__ = "GB300SPECTSystemMatrix"
    return GB300SPECTSystemMatrix
