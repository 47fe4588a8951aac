"""pytomography_gb300 — GB300-native drop-in for PyTomography's projector hot path.

Module layout mirrors the reference package so that switching is an import change:
``metadata.SPECT``, ``metadata.PET``, ``transforms.SPECT``, ``projectors.SPECT``,
``projectors.PET``, ``likelihoods``, ``priors``, ``algorithms``.  The arithmetic runs in
hand-written sm_103a CUDA behind a C ABI (``include/gbtomo.h``); there is no CPU path.

Global configuration mirrors ``src/pytomography/__init__.py:15-40``.
"""
from __future__ import annotations

import torch

__version__ = "0.1.0"

device = torch.device("cuda")
dtype = torch.float32
delta = 1e-11
verbose = False


def set_dtype(dt):
    """Only float32 is implemented by the CUDA kernels (the reference default)."""
    global dtype
    if dt != torch.float32:
        raise NotImplementedError("the GB300 kernels compute in float32 only")
    dtype = dt


def set_device(d):
    global device
    device = torch.device(d)


def set_verbose(b: bool):
    global verbose
    verbose = b


def release_pool_memory() -> None:
    """Return the device memory that destroyed plans left reserved in the library's pool
    (up to 16 GiB is kept for the next plan) to the driver, e.g. before PyTorch needs it."""
    from . import _lib
    _lib.check(_lib.load().gb_release_pool_memory())
