"""ctypes binding of ``libgbtomo.so`` (declarations in ``include/gbtomo.h``).

The library is built in-tree by ``pytomography_gb300/build.py``.  There is no CPU
fallback: when the library is missing, or no CUDA device is present, the projector
classes raise.
"""
from __future__ import annotations

import ctypes
import os

import torch

from . import build as _build

c_int = ctypes.c_int32
c_float = ctypes.c_float
c_void_p = ctypes.c_void_p
c_char_p = ctypes.c_char_p


class SpectDesc(ctypes.Structure):
    _fields_ = [
        ("nx", c_int), ("ny", c_int), ("nz", c_int),
        ("dx", c_float), ("dy", c_float), ("dz", c_float),
        ("n_angles", c_int),
        ("theta_fwd", c_void_p), ("theta_bwd", c_void_p), ("lin", c_void_p),
        ("mu", c_void_p),
        ("order", c_char_p),
        ("psf_2d", c_int), ("psf_n_groups", c_int), ("psf_group", c_void_p),
        ("psf_k", c_int), ("psf_taps_r", c_void_p), ("psf_taps_z", c_void_p),
        ("psf_trunc_rel", c_float),
        ("no_pad", c_int),
        ("psf_k_min", c_int),
    ]


class SpectTuning(ctypes.Structure):
    _fields_ = [("fwd_tpb", c_int), ("fwd_zt", c_int), ("fwd_items", c_int), ("b1_zt", c_int),
                ("b1_items", c_int), ("fwd_variant", c_int), ("osem_split", c_int)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class RdpDesc(ctypes.Structure):
    _fields_ = [("beta", c_float), ("gamma", c_float), ("delta", c_float),
                ("fov_scale", c_void_p)]


class PetDesc(ctypes.Structure):
    _fields_ = [
        ("nx", c_int), ("ny", c_int), ("nz", c_int),
        ("vx", c_float), ("vy", c_float), ("vz", c_float),
        ("ox", c_float), ("oy", c_float), ("oz", c_float),
        ("n_det", c_int), ("lut", c_void_p),
        ("tof", c_int), ("tof_num_bins", c_int), ("tof_bin_width", c_float),
        ("tof_sigma", c_float), ("tof_center_offset", c_float), ("tof_n_sigmas", c_float),
        ("n_events", ctypes.c_int64), ("events", c_void_p),
    ]


class PetSinoDesc(ctypes.Structure):
    _fields_ = [
        ("nx", c_int), ("ny", c_int), ("nz", c_int),
        ("vx", c_float), ("vy", c_float), ("vz", c_float),
        ("ox", c_float), ("oy", c_float), ("oz", c_float),
        ("n_angles", c_int), ("n_radial", c_int), ("n_planes", c_int),
        ("det_xy", c_void_p), ("plane_z", c_void_p),
        ("tof", c_int), ("tof_num_bins", c_int), ("tof_bin_width", c_float),
        ("tof_sigma", c_float), ("tof_center_offset", c_float), ("tof_n_sigmas", c_float),
    ]


_LIB = None

# (name, restype, argtypes) of every exported symbol declared in include/gbtomo.h
SIGNATURES = [
    ("gb_last_error", c_char_p, []),
    ("gb_version", c_char_p, []),
    ("gb_release_pool_memory", c_int, []),
    ("gb_spect_plan_create", c_int, [ctypes.POINTER(SpectDesc), ctypes.POINTER(c_void_p)]),
    ("gb_spect_plan_destroy", c_int, [c_void_p]),
    ("gb_spect_set_subsets", c_int, [c_void_p, c_int]),
    ("gb_spect_device_status", c_int, [c_void_p, ctypes.POINTER(c_int)]),
    ("gb_spect_clear_device_status", c_int, [c_void_p]),
    ("gb_spect_set_debug", c_int, [c_void_p, c_int, c_int]),
    ("gb_inject_fault", c_int, [c_char_p, c_int]),
    ("gb_spect_subset_size", c_int, [c_void_p, c_int]),
    ("gb_spect_set_subset_lists", c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    ("gb_starguide_window", c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_void_p,
                                    c_void_p, c_void_p]),
    ("gb_starguide_window_adjoint", c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                            c_void_p, c_void_p, c_void_p]),
    ("gb_spect_get_tuning", c_int, [c_void_p, ctypes.POINTER(SpectTuning)]),
    ("gb_spect_set_tuning", c_int, [c_void_p, ctypes.POINTER(SpectTuning)]),
    ("gb_spect_autotune", c_int, [c_void_p, c_int, c_int, ctypes.POINTER(SpectTuning), c_void_p]),
    ("gb_spect_forward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("gb_spect_backward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]),
    ("gb_spect_osem_step", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                   c_void_p, c_void_p]),
    ("gb_spect_bsrem_step", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_float, c_float, ctypes.POINTER(RdpDesc),
                                    c_float, c_int, c_void_p]),
    ("gb_spect_attenuation_apply", c_int, [c_void_p, c_int, c_int, c_int, c_float, c_void_p,
                                           c_void_p, c_void_p, c_void_p, c_void_p]),
    ("gb_spect_psf_apply", c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_int,
                                   c_void_p, c_int, c_void_p]),
    ("gb_spect_batch_create", c_int, [c_void_p, c_int, ctypes.POINTER(c_void_p)]),
    ("gb_spect_batch_destroy", c_int, [c_void_p]),
    ("gb_spect_batch_forward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("gb_spect_batch_backward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]),
    ("gb_spect_batch_osem_step", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                         c_void_p]),
    ("gb_rdp_gradient", c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_float, c_float,
                                c_float, ctypes.POINTER(RdpDesc), c_float, c_void_p]),
    ("gb_rdp_hessian_vector", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_float,
                                      c_float, c_float, ctypes.POINTER(RdpDesc), c_float,
                                      c_void_p]),
    ("gb_pet_plan_create", c_int, [ctypes.POINTER(PetDesc), ctypes.POINTER(c_void_p)]),
    ("gb_pet_plan_destroy", c_int, [c_void_p]),
    ("gb_pet_set_subsets", c_int, [c_void_p, c_int]),
    ("gb_pet_forward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("gb_pet_backward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("gb_pet_set_deterministic", c_int, [c_void_p, c_int]),
    ("gb_pet_lor_forward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]),
    ("gb_pet_sensitivity", c_int, [c_void_p, c_void_p, ctypes.c_int64, c_void_p, c_void_p,
                                   c_float, c_void_p, c_void_p]),
    ("gb_pet_osem_step", c_int, [c_void_p, c_void_p, c_void_p, ctypes.c_int64, c_void_p,
                                 c_void_p, c_int, c_void_p]),
    ("gb_pet_sino_plan_create", c_int, [ctypes.POINTER(PetSinoDesc), ctypes.POINTER(c_void_p)]),
    ("gb_pet_sino_plan_destroy", c_int, [c_void_p]),
    ("gb_pet_sino_set_subsets", c_int, [c_void_p, c_int]),
    ("gb_pet_sino_subset_size", c_int, [c_void_p, c_int]),
    ("gb_pet_sino_forward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]),
    ("gb_pet_sino_backward", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]),
    ("gb_pet_sino_atten", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    ("gb_filter3d", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_int,
                            c_void_p, c_int, c_void_p, c_int, c_void_p]),
    ("gb_kem_apply", c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                             c_void_p]),
    ("gb_pet_lm_to_sino", c_int, [c_void_p, ctypes.c_int64, c_int, c_void_p, c_void_p, c_void_p,
                                  c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_void_p,
                                  c_void_p]),
]


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the CUDA library; raises if it cannot."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing and _build.needs_build():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libgbtomo.so not built ({path}); run pytomography_gb300.build")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != 0:
        msg = _LIB.gb_last_error().decode() if _LIB is not None else ""
        raise RuntimeError(f"gbtomo error {status}: {msg}")


def require_cuda(t: torch.Tensor, name: str) -> None:
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor (no CPU path exists)")
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def stream_handle(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor | None):
    return None if t is None else ctypes.c_void_p(t.data_ptr())
