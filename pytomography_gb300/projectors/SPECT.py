"""Drop-in ``SPECTSystemMatrix`` running the fused sm_103a projector.

Mirror of src/pytomography/projectors/SPECT/spect_system_matrix.py:15-201.  The
constructor takes the reference's arguments; the obj2obj plugins
(``SPECTAttenuationTransform``, ``SPECTPSFTransform``) are lowered into one CUDA plan
(geometry tables, attenuation factors per angle, per-plane PSF taps) and every projection
is a few kernel launches through ``libgbtomo.so``.  Unknown transforms raise; there is no
CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib, geometry
from ..transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
from .system_matrix import SystemMatrix


# PSF tap counts the fused kernels are compiled for (a plan's taps are zero-padded to the
# smallest that holds them)
PSF_BUCKETS = (7, 11, 15, 21, 25, 29, 37, 45)


class SPECTSystemMatrix(SystemMatrix):
    """Rotate+sum SPECT system matrix.

    Args:
        obj2obj_transforms: attenuation and/or PSF plugins, in application order.
        proj2proj_transforms: must be empty (no proj2proj plugin is on this path).
        object_meta, proj_meta: SPECT metadata.
        object_initial_based_on_camera_path: zero voxels the camera path never sees.
        psf_trunc_rel: PSF taps below this fraction of a plane's largest tap are skipped
            (default 1e-7: changes projections by well under 1e-6 relative; 0 keeps every
            tap of the reference's kernel).
        autotune: time the kernels' tile candidates on the device whenever the subsets
            change (results are cached per geometry for the process) instead of using the
            shared-memory-derived defaults.  Tiles change no result beyond the order of
            floating-point sums.
        check_device_status: after every projector call, read the plan's device error
            word (a synchronous read) and raise if a kernel gave up on a bounded wait.
    """

    _tuning_cache: dict = {}

    def __init__(self, obj2obj_transforms, proj2proj_transforms, object_meta, proj_meta,
                 object_initial_based_on_camera_path: bool = False,
                 psf_trunc_rel: float = 1e-7, autotune: bool = False,
                 check_device_status: bool = False, _no_pad: bool = False,
                 _psf_k_min: int = 0) -> None:
        if proj2proj_transforms:
            raise NotImplementedError("proj2proj transforms are not part of the fused path")
        super().__init__(object_meta, proj_meta, obj2obj_transforms, proj2proj_transforms)
        self.object_initial_based_on_camera_path = object_initial_based_on_camera_path
        self.psf_trunc_rel = float(psf_trunc_rel)
        self.autotune_enabled = bool(autotune)
        self.check_device_status = bool(check_device_status)
        self._no_pad = bool(_no_pad)  # unpadded rotation frame (the StarGuide projector)
        self._psf_k_min = int(_psf_k_min)  # smallest PSF tap bucket (plans batched together)
        self._lists_epoch = 0  # bumped whenever the plan's subset or tile lists change
        self._plan = None
        self._lib = _lib.load()
        self._build_plan()
        self.subset_indices_array = None
        self.n_subsets = 1

    # ------------------------------------------------------------ plan
    def _build_plan(self) -> None:
        om, pm = self.object_meta, self.proj_meta
        nx, ny, nz = (int(s) for s in om.shape)
        if nx != ny:
            raise ValueError("rotate+sum needs Lx == Ly")
        if tuple(pm.shape[1:]) != (ny, nz):
            raise ValueError(f"projection shape {pm.shape[1:]} does not match object {om.shape}")
        if not torch.cuda.is_available():
            raise RuntimeError("SPECTSystemMatrix needs a CUDA device (no CPU path)")
        self.device = torch.device("cuda", torch.cuda.current_device())
        n = pm.num_projections
        Lp = nx if self._no_pad else om.padded_shape[0]
        for t in self.obj2obj_transforms:
            if getattr(t, "assume_padded", True) == self._no_pad:
                raise NotImplementedError(
                    "transforms must be configured for the system matrix's frame "
                    "(assume_padded=True for SPECTSystemMatrix, False for StarGuide)")
        angles = pm.angles.to(torch.float32).cpu()
        # forward rotation: RotationTransform.backward(obj, 270 - beta) -> rotate(beta - 270);
        # back-projection rotation: RotationTransform.forward(obj, 270 - beta).  One batched
        # call (every matrix is computed on its own, so the rows are those of two calls).
        both = geometry.rotation_theta(torch.cat([-(270 - angles), 270 - angles]), Lp)
        self._theta_fwd, self._theta_bwd = both[:n].contiguous(), both[n:].contiguous()
        self._lin = geometry.base_grid(Lp)
        order = ""
        mu = None
        psf_tables = None
        self._transform_order = []
        for t in self.obj2obj_transforms:
            if isinstance(t, SPECTAttenuationTransform):
                order += "a"
                mu = t.attenuation_map.to(self.device, torch.float32).contiguous()
            elif isinstance(t, SPECTPSFTransform):
                order += "p"
                psf_tables = t
            else:
                raise NotImplementedError(
                    f"transform {type(t).__name__} has no fused GB300 implementation")
        if order.count("a") > 1 or order.count("p") > 1:
            raise NotImplementedError("at most one attenuation and one PSF transform")
        self._order = order
        self._mu = mu
        desc = _lib.SpectDesc()
        desc.nx, desc.ny, desc.nz = nx, ny, nz
        desc.dx, desc.dy, desc.dz = (float(v) for v in om.dr)
        desc.n_angles = n
        keep = []

        def host(t, dt=torch.float32):
            a = t.to(dt).contiguous().cpu().numpy()
            keep.append(a)
            return a.ctypes.data_as(ctypes.c_void_p)

        desc.theta_fwd = host(self._theta_fwd)
        desc.theta_bwd = host(self._theta_bwd)
        desc.lin = host(self._lin)
        desc.mu = None if mu is None else ctypes.c_void_p(mu.data_ptr())
        desc.order = order.encode()
        if psf_tables is not None:
            radii = psf_tables.radii_unique
            group = np.array([radii.index(float(r)) for r in pm.radii], dtype=np.int32)
            k = 1
            two_d = True
            for r in radii:
                wr, wz = psf_tables.tables[r]
                k = max(k, wr.shape[1], 0 if wz is None else wz.shape[1])
                two_d = wz is not None
            tr = np.zeros((len(radii), Lp, k), np.float32)
            tz = np.zeros((len(radii), Lp, k), np.float32)
            for gi, r in enumerate(radii):
                wr, wz = psf_tables.tables[r]
                o = (k - wr.shape[1]) // 2
                tr[gi, :, o:o + wr.shape[1]] = wr.numpy()
                if wz is not None:
                    o = (k - wz.shape[1]) // 2
                    tz[gi, :, o:o + wz.shape[1]] = wz.numpy()
            keep.extend([tr, tz, group])
            desc.psf_2d = 1 if two_d else 0
            desc.psf_n_groups = len(radii)
            desc.psf_group = group.ctypes.data_as(ctypes.c_void_p)
            desc.psf_k = k
            desc.psf_taps_r = tr.ctypes.data_as(ctypes.c_void_p)
            desc.psf_taps_z = tz.ctypes.data_as(ctypes.c_void_p)
            desc.psf_trunc_rel = self.psf_trunc_rel
            self._psf_k = k
        else:
            self._psf_k = 1
        desc.no_pad = 1 if self._no_pad else 0
        desc.psf_k_min = self._psf_k_min
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            torch.cuda.synchronize()
            _lib.check(self._lib.gb_spect_plan_create(ctypes.byref(desc), ctypes.byref(handle)))
        self._plan = handle

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and self._lib is not None:
            try:
                self._lib.gb_spect_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    def device_status(self) -> int:
        """Device error word of the plan (0 = no kernel gave up on a bounded wait)."""
        code = ctypes.c_int32(0)
        _lib.check(self._lib.gb_spect_device_status(self._plan, ctypes.byref(code)))
        return int(code.value)

    def raise_on_device_error(self) -> None:
        """Raise (and reset the error word) when a kernel of this plan gave up on a
        bounded wait; its outputs since the last check are then invalid."""
        code = self.device_status()
        if code:
            _lib.check(self._lib.gb_spect_clear_device_status(self._plan))
            raise RuntimeError(f"gbtomo device error {code}: a projector kernel gave up waiting "
                               "for its attenuation copies; outputs since the last check are "
                               "invalid")

    @property
    def psf_bucket(self) -> int:
        """Tap count the plan's PSF kernels are compiled for (0 without PSF)."""
        if "p" not in self._order:
            return 0
        k = max(self._psf_k, self._psf_k_min)
        return next(b for b in PSF_BUCKETS if k <= b)

    def _rebuild_plan(self, psf_k_min: int) -> None:
        """Create the plan again with at least ``psf_k_min`` taps per PSF kernel (the same
        projections: the extra taps are zero), keeping the current subsets."""
        old = self._plan
        self._psf_k_min = int(psf_k_min)
        self._build_plan()
        if old is not None:
            self._lib.gb_spect_plan_destroy(old)
        if self.subset_indices_array is not None and self.n_subsets > 1:
            _lib.check(self._lib.gb_spect_set_subsets(self._plan, int(self.n_subsets)))
        self._lists_epoch += 1

    def _after_call(self) -> None:
        if self.check_device_status:
            self.raise_on_device_error()

    # ------------------------------------------------------------ subsets
    def set_n_subsets(self, n_subsets: int) -> None:
        if self.subset_indices_array is not None and int(n_subsets) == self.n_subsets:
            return  # the same split: indices and the plan's work lists are unchanged
        indices = torch.arange(self.proj_meta.shape[0]).to(torch.long).to(self.device)
        self.subset_indices_array = [indices[i::n_subsets] for i in range(n_subsets)]
        self.n_subsets = n_subsets
        _lib.check(self._lib.gb_spect_set_subsets(self._plan, int(n_subsets)))
        self._lists_epoch += 1
        if self.autotune_enabled:
            self.autotune()

    # ------------------------------------------------------------ tiles
    def _tuning_key(self, subset_idx):
        props = torch.cuda.get_device_properties(self.device)
        return (props.name, tuple(int(v) for v in self.object_meta.shape),
                tuple(float(v) for v in self.object_meta.dr), self._order, self.psf_bucket,
                int(self.proj_meta.num_projections), int(self.n_subsets),
                self._n_sel(subset_idx))

    def get_tuning(self) -> dict:
        t = _lib.SpectTuning()
        _lib.check(self._lib.gb_spect_get_tuning(self._plan, ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, **fields) -> None:
        t = _lib.SpectTuning(**{**self.get_tuning(), **fields})
        _lib.check(self._lib.gb_spect_set_tuning(self._plan, ctypes.byref(t)))
        self._lists_epoch += 1

    def autotune(self, subset_idx: int | None = 0, reps: int = 3) -> dict:
        """Pick the fastest kernel tiles for this geometry (gb_spect_autotune), timing
        the projections of ``subset_idx`` (the first subset by default, all angles when
        there are no subsets); repeated geometries reuse the first result."""
        if self.n_subsets <= 1:
            subset_idx = None
        key = self._tuning_key(subset_idx)
        hit = SPECTSystemMatrix._tuning_cache.get(key)
        if hit is not None:
            self.set_tuning(**hit)
            return dict(hit)
        out = _lib.SpectTuning()
        self._lists_epoch += 1
        with torch.cuda.device(self.device):
            torch.cuda.synchronize()
            _lib.check(self._lib.gb_spect_autotune(
                self._plan, self._subset_code(subset_idx), int(reps), ctypes.byref(out),
                _lib.stream_handle(self.device)))
            torch.cuda.synchronize()
        SPECTSystemMatrix._tuning_cache[key] = out.as_dict()
        return out.as_dict()

    def get_projection_subset(self, projections: torch.Tensor, subset_idx: int) -> torch.Tensor:
        return projections[..., self.subset_indices_array[subset_idx], :, :]

    def get_weighting_subset(self, subset_idx: int | None) -> float:
        if subset_idx is None:
            return 1
        return len(self.subset_indices_array[subset_idx]) / self.proj_meta.num_projections

    def _subset_code(self, subset_idx) -> int:
        if subset_idx is None:
            return -1
        if self.subset_indices_array is None:
            raise RuntimeError("set_n_subsets must be called before using subset indices")
        return int(subset_idx)

    def _n_sel(self, subset_idx) -> int:
        return self.proj_meta.num_projections if subset_idx is None else \
            len(self.subset_indices_array[subset_idx])

    # ------------------------------------------------------------ projectors
    def _object_in(self, object: torch.Tensor) -> torch.Tensor:
        obj = object.to(self.device, torch.float32)
        if tuple(obj.shape) != tuple(self.object_meta.shape):
            raise ValueError(f"object shape {tuple(obj.shape)} != {tuple(self.object_meta.shape)}")
        return obj.contiguous()

    def forward(self, object: torch.Tensor, subset_idx: int | None = None) -> torch.Tensor:
        """H_m f -> [n_sel, Ly, Lz] (spect_system_matrix.py:120-157)."""
        obj = self._object_in(object)
        code = self._subset_code(subset_idx)
        out = torch.empty((self._n_sel(subset_idx), *self.proj_meta.shape[1:]),
                          device=self.device, dtype=torch.float32)
        _lib.check(self._lib.gb_spect_forward(self._plan, _lib.ptr(obj), _lib.ptr(out), code,
                                              _lib.stream_handle(self.device)))
        self._after_call()
        return out

    def _backward(self, proj: torch.Tensor, subset_idx, adjoint: int) -> torch.Tensor:
        code = self._subset_code(subset_idx)
        p = proj.to(self.device, torch.float32).contiguous()
        exp = (self._n_sel(subset_idx), *self.proj_meta.shape[1:])
        if tuple(p.shape) != exp:
            raise ValueError(f"projection shape {tuple(p.shape)} != {exp}")
        out = torch.empty(tuple(self.object_meta.shape), device=self.device, dtype=torch.float32)
        _lib.check(self._lib.gb_spect_backward(self._plan, _lib.ptr(p), _lib.ptr(out), code,
                                               adjoint, _lib.stream_handle(self.device)))
        self._after_call()
        return out

    def backward(self, proj: torch.Tensor, subset_idx: int | None = None) -> torch.Tensor:
        """Reference back-projector (spect_system_matrix.py:159-201)."""
        return self._backward(proj, subset_idx, 0)

    def backward_adjoint(self, proj: torch.Tensor, subset_idx: int | None = None) -> torch.Tensor:
        """Exact transpose of :meth:`forward` (same bilinear taps, scattered)."""
        return self._backward(proj, subset_idx, 1)

    def compute_normalization_factor(self, subset_idx: int | None = None) -> torch.Tensor:
        n = self._n_sel(subset_idx)
        ones = torch.ones((n, *self.proj_meta.shape[1:]), device=self.device)
        return self.backward(ones, subset_idx)

    def compute_normalization_factors(self) -> list:
        """H_m^T 1 of every subset of the current split, in subset order: the values of
        ``compute_normalization_factor(m)`` for each m, from one buffer of ones and one
        back-projection call per subset."""
        if self.subset_indices_array is None:
            return [self.compute_normalization_factor(None)]
        n_max = max(len(ix) for ix in self.subset_indices_array)
        ones = torch.ones((n_max, *self.proj_meta.shape[1:]), device=self.device)
        st = _lib.stream_handle(self.device)
        outs = []
        for k in range(len(self.subset_indices_array)):
            out = torch.empty(tuple(self.object_meta.shape), device=self.device,
                              dtype=torch.float32)
            # the first n_sel(k) rows of the buffer are subset k's projection of ones
            _lib.check(self._lib.gb_spect_backward(self._plan, _lib.ptr(ones), _lib.ptr(out),
                                                   k, 0, st))
            outs.append(out)
        self._after_call()
        return outs

    # ------------------------------------------------------------ fused updates
    def osem_step(self, object: torch.Tensor, projections: torch.Tensor,
                  additive: torch.Tensor | None, norm_bp: torch.Tensor,
                  subset_idx: int | None, predicted: torch.Tensor | None = None) -> None:
        """In-place fused OSEM sub-iteration (see gb_spect_osem_step)."""
        _lib.require_cuda(object, "object")
        g = projections.to(self.device, torch.float32).contiguous()
        s = None if additive is None else additive.to(self.device, torch.float32).contiguous()
        nb = norm_bp.contiguous()
        _lib.check(self._lib.gb_spect_osem_step(
            self._plan, _lib.ptr(object), _lib.ptr(g), _lib.ptr(s), _lib.ptr(nb),
            self._subset_code(subset_idx), _lib.ptr(predicted), _lib.stream_handle(self.device)))
        self._after_call()

    def bsrem_step(self, object_in, object_out, projections, additive, norm_bp, norm_bp_sum,
                   relax: float, subset_weight: float, prior=None, floor_value: float = 1e-4,
                   subset_idx: int | None = None) -> None:
        g = projections.contiguous()
        s = None if additive is None else additive.contiguous()
        rd = None
        if prior is not None:
            rd = _lib.RdpDesc(float(prior.beta), float(prior.gamma), float(prior.delta),
                              None if prior.FOV_scale is None
                              else ctypes.c_void_p(prior.FOV_scale.data_ptr()))
        _lib.check(self._lib.gb_spect_bsrem_step(
            self._plan, _lib.ptr(object_in), _lib.ptr(object_out), _lib.ptr(g), _lib.ptr(s),
            _lib.ptr(norm_bp), _lib.ptr(norm_bp_sum), float(relax), float(subset_weight),
            None if rd is None else ctypes.byref(rd), float(floor_value),
            self._subset_code(subset_idx), _lib.stream_handle(self.device)))

    # ------------------------------------------------------------ initial object
    def _get_object_initial(self, device=None) -> torch.Tensor:
        """Ones, optionally zeroed outside the camera path (spect_system_matrix.py:38-56)."""
        dev = self.device if device is None else device
        obj = torch.ones(tuple(self.object_meta.shape), device=dev)
        if not self.object_initial_based_on_camera_path:
            return obj
        nx = self.object_meta.shape[0]
        for i in range(len(self.proj_meta.angles)):
            cutoff = int(np.ceil(nx / 2 - self.proj_meta.radii[i] / self.object_meta.dr[0]))
            if cutoff < 0:
                continue
            cut = torch.ones(tuple(self.object_meta.shape), device=self.device)
            cut[:cutoff] = 0
            obj *= self._rotate_unpadded(cut, -(270 - float(self.proj_meta.angles[i]))).to(dev)
        return obj

    def _rotate_unpadded(self, x: torch.Tensor, angle: float) -> torch.Tensor:
        """pad -> kornia-convention rotation -> unpad (setup-time helper, not the hot path)."""
        pad = self.object_meta.pad_size
        xp = torch.nn.functional.pad(x, [0, 0, pad, pad, pad, pad])
        Lp = xp.shape[0]
        theta = geometry.rotation_theta(torch.tensor([angle]), Lp).view(1, 2, 3).to(x.device)
        img = xp.permute(2, 0, 1).unsqueeze(0)
        grid = torch.nn.functional.affine_grid(theta, list(img.shape), align_corners=True)
        r = torch.nn.functional.grid_sample(img, grid, mode="bilinear", padding_mode="zeros",
                                            align_corners=True)
        r = r.squeeze(0).permute(1, 2, 0)
        return r[pad:-pad, pad:-pad, :]


class StarGuideSystemMatrix(SystemMatrix):
    """StarGuide SPECT system matrix (projectors/SPECT/starguide_system_matrix.py:12-230).

    Every projection is one detector at an angle, with a radius (PSF), an offset along y
    and an acquisition time.  Its forward projection is the rotate -> attenuate -> PSF ->
    sum projection of the object in the unpadded frame (transforms configured with
    ``assume_padded=False``), translated along y by offset / dx, cropped to the detector
    window and scaled by time / 1000.  Here the projection runs on the fused SPECT kernels
    (one plan entry per detector, no padding) and the window on ``gb_starguide_window``;
    the back projection pads, translates back and runs the reference back-projector.
    Subsets are whole angle groups: subset k holds the detectors of the sorted unique
    angles k, k + n, ... (:166-179).
    """

    def __init__(self, object_meta, proj_meta, obj2obj_transforms=None,
                 proj2proj_transforms=None) -> None:
        from ..metadata.SPECT import SPECTProjMeta
        if proj2proj_transforms:
            raise NotImplementedError("proj2proj transforms are not part of the fused path")
        self.object_meta = object_meta
        self.proj_meta = proj_meta
        self.obj2obj_transforms = list(obj2obj_transforms or [])
        self.proj2proj_transforms = []
        n = int(proj_meta.num_projections)
        nx, ny, nz = (int(v) for v in object_meta.shape)
        angles = torch.as_tensor(proj_meta.angles, dtype=torch.float32).cpu()
        radii = [0.0] * n if proj_meta.radii is None else [float(r) for r in proj_meta.radii]
        inner = SPECTProjMeta((ny, nz), list(object_meta.dr[:2]), angles.tolist(), radii=radii)
        self._H = SPECTSystemMatrix(self.obj2obj_transforms, [], object_meta, inner, _no_pad=True)
        self.device = self._H.device
        self._lib = self._H._lib
        self.times = torch.as_tensor(proj_meta.times, dtype=torch.float32).reshape(-1, 1, 1) / 1e3
        offsets = torch.as_tensor(proj_meta.offsets, dtype=torch.float32)
        self._shift = (offsets / float(object_meta.dx)).to(self.device).contiguous()
        self._scale = self.times.reshape(-1).to(self.device).contiguous()
        self._width = int(proj_meta.shape[1])
        self.subset_indices_array = None
        self.n_subsets = 1

    # ------------------------------------------------------------ subsets
    def set_n_subsets(self, n_subsets: int) -> None:
        angles = torch.as_tensor(self.proj_meta.angles)
        groups = [torch.where(angles == a)[0] for a in torch.unique(angles)]
        lists = [torch.cat(groups[i::n_subsets]) for i in range(n_subsets)]
        self.subset_indices_array = [ix.to(self.device) for ix in lists]
        self.n_subsets = n_subsets
        flat = torch.cat(lists).to(torch.int32).numpy()
        counts = np.array([len(ix) for ix in lists], np.int32)
        _lib.check(self._lib.gb_spect_set_subset_lists(
            self._H._plan, int(n_subsets), flat.ctypes.data_as(ctypes.c_void_p),
            counts.ctypes.data_as(ctypes.c_void_p)))
        self._H.subset_indices_array = self.subset_indices_array
        self._H.n_subsets = n_subsets

    def get_projection_subset(self, projections, subset_idx):
        return projections[..., self.subset_indices_array[subset_idx], :, :]

    def get_weighting_subset(self, subset_idx):
        if subset_idx is None:
            return 1
        return len(self.subset_indices_array[subset_idx]) / self.proj_meta.num_projections

    def _rows(self, subset_idx):
        if subset_idx is None:
            return torch.arange(self.proj_meta.num_projections, device=self.device)
        return self.subset_indices_array[subset_idx]

    # ------------------------------------------------------------ projectors
    def forward(self, object, subset_idx=None):
        full = self._H.forward(object, subset_idx)
        rows = self._rows(subset_idx)
        shift = self._shift[rows].contiguous()
        scale = self._scale[rows].contiguous()
        n, ny, nz = full.shape
        out = torch.empty((n, self._width, nz), device=self.device)
        _lib.check(self._lib.gb_starguide_window(_lib.ptr(full), _lib.ptr(out), n, ny, nz,
                                                 self._width, _lib.ptr(shift), _lib.ptr(scale),
                                                 _lib.stream_handle(self.device)))
        return out

    def backward(self, proj, subset_idx=None):
        p = proj.to(self.device, torch.float32).contiguous()
        rows = self._rows(subset_idx)
        shift = self._shift[rows].contiguous()
        scale = self._scale[rows].contiguous()
        n, _, nz = p.shape
        ny = int(self.object_meta.shape[1])
        full = torch.empty((n, ny, nz), device=self.device)
        _lib.check(self._lib.gb_starguide_window_adjoint(_lib.ptr(p), _lib.ptr(full), n, ny, nz,
                                                         self._width, _lib.ptr(shift),
                                                         _lib.ptr(scale),
                                                         _lib.stream_handle(self.device)))
        return self._H.backward(full, subset_idx)

    def compute_normalization_factor(self, subset_idx=None):
        ones = torch.ones(tuple(self.proj_meta.shape), device=self.device)
        if subset_idx is not None:
            ones = self.get_projection_subset(ones, subset_idx)
        return self.backward(ones, subset_idx)

    def _get_object_initial(self, device=None):
        return torch.ones(tuple(self.object_meta.shape), device=self.device if device is None
                          else device)

    def _get_prior_FOV_scale(self):
        return torch.ones(tuple(self.object_meta.shape), device=self.device)
