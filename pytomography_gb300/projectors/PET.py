"""Drop-in ``PETLMSystemMatrix`` on the sm_103a TOF Joseph listmode kernels.

Mirror of src/pytomography/projectors/PET/petlm_system_matrix.py:11-363.  Events and the
scanner LUT are uploaded once and stay resident on the GPU (the reference gathers LUT rows
on the CPU and copies them to the device on every call); subsets ``i::n`` are addressed
by stride inside the kernels, so no gather copies are made.  The sensitivity image
generates every crystal pair on the device instead of materialising torch.combinations.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib
from .system_matrix import SystemMatrix


class PETLMSystemMatrix(SystemMatrix):
    def __init__(self, object_meta, proj_meta, obj2obj_transforms=None,
                 attenuation_map: torch.Tensor | None = None,
                 scale_projection_by_sensitivity: bool = False, N_splits: int = 1,
                 FOV_scale_enabled: bool = True, device=None,
                 compute_sensitivity: bool = True) -> None:
        if not torch.cuda.is_available():
            raise RuntimeError("PETLMSystemMatrix needs a CUDA device (no CPU path)")
        # object-space transforms (e.g. GaussianFilter as the resolution model) run before
        # forward projection and after back projection (petlm_system_matrix.py:258-260,
        # 359-361); they disable the fused OSEM step
        super().__init__(object_meta, proj_meta, obj2obj_transforms or [], [])
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.output_device = self.device if device is None else torch.device(device)
        self.TOF = proj_meta.tof_meta is not None
        self.object_origin = (-np.array(object_meta.shape) / 2 + 0.5) * np.array(object_meta.dr)
        self.proj_meta.detector_ids = self.proj_meta.detector_ids.cpu()
        self.proj_meta.scanner_lut = self.proj_meta.scanner_lut.cpu()
        self.attenuation_map = attenuation_map
        self.N_splits = N_splits
        self.scale_projection_by_sensitivity = scale_projection_by_sensitivity
        self.FOV_scale_enabled = FOV_scale_enabled
        self._lib = _lib.load()
        self._build_plan()
        self.subset_indices_array = None
        self.n_subsets = 1
        if compute_sensitivity:
            self.norm_BP = self._backward_full()
            self.norm_BP[self.norm_BP < 1e-7] = 1e7
        else:
            self.norm_BP = None

    def _build_plan(self):
        om, pm = self.object_meta, self.proj_meta
        d = _lib.PetDesc()
        d.nx, d.ny, d.nz = (int(s) for s in om.shape)
        d.vx, d.vy, d.vz = (float(v) for v in om.dr)
        d.ox, d.oy, d.oz = (float(v) for v in self.object_origin)
        lut = pm.scanner_lut.to(torch.float32).contiguous().numpy()
        d.n_det = lut.shape[0]
        d.lut = lut.ctypes.data_as(ctypes.c_void_p)
        ncol = 3 if self.TOF else 2
        ids = pm.detector_ids[:, :ncol].to(torch.int32).contiguous()
        self._ids_dev = ids.to(self.device)
        d.n_events = ids.shape[0]
        d.events = ctypes.c_void_p(self._ids_dev.data_ptr())
        if self.TOF:
            t = pm.tof_meta
            d.tof = 1
            d.tof_num_bins = int(t.num_bins)
            d.tof_bin_width = float(t.bin_width)
            d.tof_sigma = float(t.sigma)
            d.tof_center_offset = float(t.center_offset)
            d.tof_n_sigmas = float(t.n_sigmas)
        h = ctypes.c_void_p()
        torch.cuda.synchronize()
        _lib.check(self._lib.gb_pet_plan_create(ctypes.byref(d), ctypes.byref(h)))
        self._plan = h
        self._keep = (lut, ids)

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and getattr(self, "_lib", None) is not None:
            try:
                self._lib.gb_pet_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    # ------------------------------------------------------------ FOV helpers
    def _z_fov(self):
        lut_z = self.proj_meta.scanner_lut[:, 2]
        nzv = self.object_meta.shape[-1]
        zmin = (nzv - 1) / 2 + float(lut_z.min()) / self.object_meta.dr[-1]
        zmax = (nzv - 1) / 2 + float(lut_z.max()) / self.object_meta.dr[-1]
        return zmin, zmax

    def _get_object_initial(self, device=None):
        zmin, zmax = self._z_fov()
        zmin, zmax = max(0, zmin), max(0, zmax)
        obj = torch.ones(tuple(self.object_meta.shape)).to(self.device if device is None else device)
        obj[:, :, :int(np.ceil(zmin))] = 0
        obj[:, :, int(np.floor(zmax)):] = 0
        return obj

    def _get_prior_FOV_scale(self):
        if not self.FOV_scale_enabled:
            return torch.ones(tuple(self.object_meta.shape)).to(self.device)
        zmin, zmax = self._z_fov()
        zmid = (zmin + zmax) / 2
        z = torch.arange(self.object_meta.shape[-1]).to(self.device)
        fov = (zmid - torch.abs(z - zmid)) / zmid
        fov[fov < 0] = 0
        return torch.ones(tuple(self.object_meta.shape)).to(self.device) * fov

    # ------------------------------------------------------------ subsets
    def set_deterministic(self, on: bool = True) -> None:
        """Back projections accumulate as 64-bit fixed-point sums (gb_pet_set_deterministic):
        bit-identical from run to run, equal to the float path to rounding."""
        _lib.check(self._lib.gb_pet_set_deterministic(self._plan, int(bool(on))))

    def set_n_subsets(self, n_subsets: int) -> None:
        idx = torch.arange(self.proj_meta.detector_ids.shape[0]).to(torch.long).cpu()
        self.subset_indices_array = [idx[i::n_subsets] for i in range(n_subsets)]
        self.n_subsets = n_subsets
        _lib.check(self._lib.gb_pet_set_subsets(self._plan, int(n_subsets)))

    def get_projection_subset(self, projections, subset_idx):
        if projections.shape[0] > 1 and subset_idx is not None:
            return projections[self.subset_indices_array[subset_idx]]
        return projections

    def get_weighting_subset(self, subset_idx):
        if subset_idx is None:
            return 1
        return len(self.subset_indices_array[subset_idx]) / self.proj_meta.detector_ids.shape[0]

    def compute_normalization_factor(self, subset_idx=None):
        frac = 1 if subset_idx is None else \
            self.subset_indices_array[subset_idx].shape[0] / self.proj_meta.detector_ids.shape[0]
        return frac * self.norm_BP.to(self.output_device)

    def _code(self, subset_idx):
        if subset_idx is None:
            return -1
        if self.subset_indices_array is None:
            raise RuntimeError("set_n_subsets must be called before using subset indices")
        return int(subset_idx)

    def _n_sel(self, subset_idx):
        return self.proj_meta.detector_ids.shape[0] if subset_idx is None else \
            len(self.subset_indices_array[subset_idx])

    # ------------------------------------------------------------ projectors
    def _weights(self, subset_idx):
        if self.proj_meta.weights is None:
            raise Exception("If scaling by sensitivity, then `weights` must be provided in the "
                            "projection metadata")
        return self.get_projection_subset(self.proj_meta.weights, subset_idx).to(self.device)

    def forward(self, object, subset_idx=None):
        for t in self.obj2obj_transforms:
            object = t.forward(object)
        img = object.to(self.device, torch.float32).contiguous()
        out = torch.empty(self._n_sel(subset_idx), device=self.device)
        _lib.check(self._lib.gb_pet_forward(self._plan, _lib.ptr(img), _lib.ptr(out),
                                            self._code(subset_idx), _lib.stream_handle(self.device)))
        if self.scale_projection_by_sensitivity:
            out = out * self._weights(subset_idx)
        return out.to(self.output_device)

    def backward(self, proj, subset_idx=None, return_norm_constant: bool = False):
        p = proj.to(self.device, torch.float32)
        if self.scale_projection_by_sensitivity:
            p = p * self._weights(subset_idx)
        p = p.contiguous()
        out = torch.empty(tuple(self.object_meta.shape), device=self.device)
        _lib.check(self._lib.gb_pet_backward(self._plan, _lib.ptr(p), _lib.ptr(out),
                                             self._code(subset_idx), _lib.stream_handle(self.device)))
        for t in self.obj2obj_transforms[::-1]:
            out = t.backward(out)
        if return_norm_constant:
            return out.to(self.output_device), self.compute_normalization_factor(subset_idx)
        return out.to(self.output_device)

    def osem_step(self, object, numerator, additive, norm_bp, subset_idx):
        """Fused listmode OSEM sub-iteration in place on ``object``."""
        if self.obj2obj_transforms:
            raise NotImplementedError("the fused listmode step has no object-space transforms")
        num = numerator.to(self.device, torch.float32).contiguous()
        s = None if additive is None else additive.to(self.device, torch.float32).contiguous()
        _lib.check(self._lib.gb_pet_osem_step(self._plan, _lib.ptr(object), _lib.ptr(num),
                                              int(num.numel()), _lib.ptr(s),
                                              _lib.ptr(norm_bp.contiguous()),
                                              self._code(subset_idx),
                                              _lib.stream_handle(self.device)))

    # ------------------------------------------------------------ sensitivity
    def _backward_full(self) -> torch.Tensor:
        """H~^T (w a + delta) over the sensitivity LOR set (petlm_system_matrix.py:112-174)."""
        pm = self.proj_meta
        pairs = None
        n_pairs = 0
        if pm.detector_ids_sensitivity is not None:
            pairs = pm.detector_ids_sensitivity[:, :2].to(torch.int32).contiguous().to(self.device)
            n_pairs = pairs.shape[0]
        w = None
        if pm.weights_sensitivity is not None:
            w = pm.weights_sensitivity.to(self.device, torch.float32).contiguous()
        mu = None
        if self.attenuation_map is not None:
            mu = self.attenuation_map.to(self.device, torch.float32).contiguous()
        out = torch.empty(tuple(self.object_meta.shape), device=self.device)
        _lib.check(self._lib.gb_pet_sensitivity(self._plan, _lib.ptr(pairs), int(n_pairs),
                                                _lib.ptr(w), _lib.ptr(mu), float(1e-11),
                                                _lib.ptr(out), _lib.stream_handle(self.device)))
        for t in self.obj2obj_transforms[::-1]:
            out = t.backward(out)
        return out


class PETSinogramSystemMatrix(SystemMatrix):
    """Sinogram PET system matrix on the sm_103a Joseph / TOF kernels.

    Mirror of src/pytomography/projectors/PET/pet_sinogram_system_matrix.py:12-296.  The
    sinogram geometry tables (transaxial crystal coordinates per (angle, radial) bin, axial
    coordinates per ring-pair plane) are uploaded once; every LOR is generated on the device
    from its sinogram index instead of materialising the xyz coordinate arrays.
    """

    def __init__(self, object_meta, proj_meta, obj2obj_transforms=None,
                 attenuation_map: torch.Tensor | None = None,
                 sinogram_sensitivity: torch.Tensor | None = None,
                 scale_projection_by_sensitivity: bool = False, N_splits: int = 1,
                 device=None) -> None:
        if not torch.cuda.is_available():
            raise RuntimeError("PETSinogramSystemMatrix needs a CUDA device (no CPU path)")
        # object-space transforms run before forward projection and after back projection
        # (pet_sinogram_system_matrix.py:202-204, 293-295)
        super().__init__(object_meta, proj_meta, obj2obj_transforms or [], [])
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.output_device = self.device if device is None else torch.device(device)
        self.object_origin = (-np.array(object_meta.shape) / 2 + 0.5) * np.array(object_meta.dr)
        self.attenuation_map = attenuation_map
        self.sinogram_sensitivity = sinogram_sensitivity
        if sinogram_sensitivity is not None:
            self.sinogram_sensitivity = sinogram_sensitivity.to(self.output_device)
        self.scale_projection_by_sensitivity = scale_projection_by_sensitivity
        self.N_splits = N_splits
        self.TOF = proj_meta.tof_meta is not None
        self.subset_indices_array = None
        self._n_subsets = 1
        self._lib = _lib.load()
        self._build_plan()

    def _build_plan(self):
        om, pm = self.object_meta, self.proj_meta
        d = _lib.PetSinoDesc()
        d.nx, d.ny, d.nz = (int(s) for s in om.shape)
        d.vx, d.vy, d.vz = (float(v) for v in om.dr)
        d.ox, d.oy, d.oz = (float(v) for v in self.object_origin)
        det = pm.detector_coordinates.to(torch.float32).cpu().contiguous().numpy()
        ring = pm.ring_coordinates.to(torch.float32).cpu().contiguous().numpy()
        d.n_angles, d.n_radial, d.n_planes = det.shape[0], det.shape[1], ring.shape[0]
        d.det_xy = det.ctypes.data_as(ctypes.c_void_p)
        d.plane_z = ring.ctypes.data_as(ctypes.c_void_p)
        if self.TOF:
            t = pm.tof_meta
            d.tof = 1
            d.tof_num_bins = int(t.num_bins)
            d.tof_bin_width = float(t.bin_width)
            d.tof_sigma = float(t.sigma)
            d.tof_center_offset = float(t.center_offset)
            d.tof_n_sigmas = float(t.n_sigmas)
        h = ctypes.c_void_p()
        torch.cuda.synchronize()
        _lib.check(self._lib.gb_pet_sino_plan_create(ctypes.byref(d), ctypes.byref(h)))
        self._plan = h

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and getattr(self, "_lib", None) is not None:
            try:
                self._lib.gb_pet_sino_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    # ------------------------------------------------------------ geometry
    def _get_xyz_sinogram_coordinates(self, subset_idx: int | None = None):
        """xyz of crystal 1 and crystal 2 of every sinogram element [n_sel*R*P, 3] (the
        kernels generate these on the fly; provided for callers of the reference API)."""
        det = self.proj_meta.detector_coordinates.cpu()
        if subset_idx is not None:
            det = det[self.subset_indices_array[subset_idx].cpu()]
        z = self.proj_meta.ring_coordinates.cpu()
        A, R, P = det.shape[0], det.shape[1], z.shape[0]
        xy1 = det[:, :, 0].reshape(A, R, 1, 2).expand(A, R, P, 2)
        xy2 = det[:, :, 1].reshape(A, R, 1, 2).expand(A, R, P, 2)
        z1 = z[:, 0].reshape(1, 1, P, 1).expand(A, R, P, 1)
        z2 = z[:, 1].reshape(1, 1, P, 1).expand(A, R, P, 1)
        return (torch.cat([xy1, z1], -1).reshape(-1, 3), torch.cat([xy2, z2], -1).reshape(-1, 3))

    def _code(self, subset_idx):
        if subset_idx is None:
            return -1
        if self.subset_indices_array is None:
            raise RuntimeError("set_n_subsets must be called before using subset indices")
        return int(subset_idx)

    def _sino_shape(self, subset_idx, tof: bool):
        n = self.proj_meta.N_angles if subset_idx is None else \
            len(self.subset_indices_array[subset_idx])
        shp = (n, *self.proj_meta.shape[1:])
        return shp + ((int(self.proj_meta.tof_meta.num_bins),) if tof else ())

    def _compute_atteunation_probability_projection(self, subset_idx) -> torch.Tensor:
        """exp(-H mu) per sinogram element (pet_sinogram_system_matrix.py:87-109)."""
        mu = self.attenuation_map.to(self.device, torch.float32).contiguous()
        out = torch.empty(self._sino_shape(subset_idx, False), device=self.device)
        _lib.check(self._lib.gb_pet_sino_atten(self._plan, _lib.ptr(mu), _lib.ptr(out),
                                               self._code(subset_idx),
                                               _lib.stream_handle(self.device)))
        return out.to(self.output_device)

    def _compute_sensitivity_sinogram(self, subset_idx=None):
        """mu eta (pet_sinogram_system_matrix.py:111-129)."""
        if self.sinogram_sensitivity is not None:
            sens = self.sinogram_sensitivity
        else:
            sens = torch.ones(self.proj_meta.shape).to(self.output_device)
        if subset_idx is not None:
            sens = self.get_projection_subset(sens, subset_idx)
        if self.attenuation_map is not None:
            sens = sens * self._compute_atteunation_probability_projection(subset_idx)
        if self.TOF:
            sens = sens.unsqueeze(-1)
        return sens

    # ------------------------------------------------------------ subsets
    def set_n_subsets(self, n_subsets: int) -> None:
        indices = torch.arange(self.proj_meta.N_angles).to(torch.long).to(self.output_device)
        self.subset_indices_array = [indices[i::n_subsets] for i in range(n_subsets)]
        self._n_subsets = n_subsets
        _lib.check(self._lib.gb_pet_sino_set_subsets(self._plan, int(n_subsets)))

    def get_projection_subset(self, projections, subset_idx):
        if subset_idx is None:
            return projections
        return projections[self.subset_indices_array[subset_idx]]

    def get_weighting_subset(self, subset_idx):
        if subset_idx is None:
            return 1
        return len(self.subset_indices_array[subset_idx]) / self.proj_meta.N_angles

    def compute_normalization_factor(self, subset_idx=None):
        """H^T mu eta, non-TOF (pet_sinogram_system_matrix.py:176-186)."""
        return self.backward(1, subset_idx, force_nonTOF=True, force_scale_by_sensitivity=True)

    # ------------------------------------------------------------ projectors
    def forward(self, object, subset_idx=None):
        for t in self.obj2obj_transforms:
            object = t.forward(object)
        img = object.to(self.device, torch.float32).contiguous()
        out = torch.empty(self._sino_shape(subset_idx, self.TOF), device=self.device)
        _lib.check(self._lib.gb_pet_sino_forward(self._plan, _lib.ptr(img), _lib.ptr(out),
                                                 self._code(subset_idx), 1 if self.TOF else 0,
                                                 _lib.stream_handle(self.device)))
        out = out.to(self.output_device)
        if self.scale_projection_by_sensitivity:
            sens = self._compute_sensitivity_sinogram(subset_idx)
            out = out * (sens if self.TOF else sens.reshape(out.shape))
        return out.squeeze()

    def backward(self, proj, subset_idx=None, force_scale_by_sensitivity: bool = False,
                 force_nonTOF: bool = False):
        tof = self.TOF and not force_nonTOF
        if force_scale_by_sensitivity or self.scale_projection_by_sensitivity:
            proj = proj * self._compute_sensitivity_sinogram(subset_idx)
        shape = self._sino_shape(subset_idx, tof)
        if not isinstance(proj, torch.Tensor):
            proj = torch.full(shape, float(proj))
        p = proj.to(self.device, torch.float32).reshape(shape).contiguous()
        out = torch.empty(tuple(self.object_meta.shape), device=self.device)
        _lib.check(self._lib.gb_pet_sino_backward(self._plan, _lib.ptr(p), _lib.ptr(out),
                                                  self._code(subset_idx), 1 if tof else 0,
                                                  _lib.stream_handle(self.device)))
        for t in self.obj2obj_transforms[::-1]:
            out = t.backward(out)
        return out


def create_sinogramSM_from_LMSM(lm_system_matrix, device="cpu"):
    """Sinogram system matrix of a listmode one's scanner (pet_sinogram_system_matrix.py:
    298-332): same object, TOF metadata and attenuation map; the sensitivity weights of the
    listmode system matrix, if any, are binned into a sensitivity sinogram."""
    from ..io.PET.shared import listmode_to_sinogram
    from ..metadata.PET import PETSinogramPolygonProjMeta
    lm = lm_system_matrix.proj_meta
    pm = PETSinogramPolygonProjMeta(lm.info, lm.tof_meta)
    sens = None
    if lm.weights_sensitivity is not None:
        idxs = torch.arange(lm.scanner_lut.shape[0]).cpu()
        pairs = torch.combinations(idxs, 2)
        sens = listmode_to_sinogram(pairs, lm.info, lm.weights_sensitivity.cpu())
    return PETSinogramSystemMatrix(lm_system_matrix.object_meta, pm,
                                   obj2obj_transforms=lm_system_matrix.obj2obj_transforms,
                                   N_splits=20, attenuation_map=lm_system_matrix.attenuation_map,
                                   sinogram_sensitivity=sens, device=device)
