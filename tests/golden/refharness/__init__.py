"""Import harness for the upstream PyTomography sources (fixture generation only).

This module is used by ``tests/golden/make_golden.py`` and nothing else.  It runs
only in a container that holds the upstream sources; the generated ``.npz``
fixtures are what travels with the repository.

PyTomography imports several packages at module import time that are not part of
the projector hot path and are not installed here (pydicom, nibabel, pandas,
h5py, uproot, rt_utils, torchrbf, fft_conv_pytorch, matplotlib, parallelproj).
They are replaced by inert placeholder modules.  One dependency is *on* the hot
path: ``kornia.geometry.transform.rotate`` (used by
``src/pytomography/utils/spatial.py:31,33`` and
``src/pytomography/transforms/shared/spatial.py:36,53``).  kornia is absent, so
:func:`kornia_rotate` restates its published algorithm (kornia >= 0.6.12, the
floor pinned in ``pyproject.toml:25``; the exact version is not pinned):

* ``get_rotation_matrix2d``: ``M = T(c) . R(angle) . S(1) . T(-c)`` with
  ``R = [[cos, sin], [-sin, cos]]``, angle in degrees converted as
  ``angle * pi / 180``, centre ``c = ((W-1)/2, (H-1)/2)``;
* ``warp_affine``: the pixel matrix is conjugated into normalised coordinates
  with ``N = [[2/(W-1), 0, -1], [0, 2/(H-1), -1], [0, 0, 1]]``
  (``N . M . N^-1``), inverted, and fed to ``F.affine_grid`` and
  ``F.grid_sample`` with bilinear interpolation, zero padding and
  ``align_corners=True``.
"""
from __future__ import annotations

import importlib.abc
import importlib.machinery
import importlib.metadata
import math
import os
import sys
import types

import torch
import torch.nn.functional as F

# the upstream ``src`` folder (the one holding the ``pytomography`` package); no default
REFERENCE_SRC = os.environ.get("PYTOMOGRAPHY_REFERENCE_SRC", "")

_ABSENT = (
    "pydicom", "rt_utils", "nibabel", "pandas", "h5py", "uproot", "torchrbf",
    "fft_conv_pytorch", "matplotlib", "parallelproj", "kornia",
)


class _Anything:
    """Placeholder object: callable, subscriptable, attribute-rich."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        return _Anything()

    def __getitem__(self, k):
        return _Anything()

    def __mro_entries__(self, bases):
        return (object,)


class _PlaceholderModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        return _Anything()


class _PlaceholderFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in _ABSENT and fullname not in sys.modules:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        mod = _PlaceholderModule(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        if module.__name__ == "kornia.geometry.transform":
            module.rotate = kornia_rotate
            module.Translate = KorniaTranslate


def kornia_rotate(tensor, angle, center=None, mode="bilinear", padding_mode="zeros",
                  align_corners=True):
    """Restatement of ``kornia.geometry.transform.rotate`` (see module docstring)."""
    B, C, H, W = tensor.shape
    dt = tensor.dtype
    angle = torch.as_tensor(angle).to(dt).reshape(-1).expand(B)
    if center is None:
        center = torch.tensor([(W - 1) / 2.0, (H - 1) / 2.0], dtype=dt).expand(B, 2)
    theta = kornia_sampling_matrix(angle, center, H, W)
    grid = F.affine_grid(theta, [B, C, H, W], align_corners=align_corners)
    return F.grid_sample(tensor, grid, mode=mode, padding_mode=padding_mode,
                         align_corners=align_corners)


class KorniaTranslate:
    """Restatement of ``kornia.geometry.transform.Translate`` (used by
    ``src/pytomography/projectors/SPECT/starguide_system_matrix.py:9,227``): the pixel
    matrix ``[[1, 0, tx], [0, 1, ty]]`` per batch element, conjugated into normalised
    coordinates like ``rotate`` and inverted, sampled with ``affine_grid`` /
    ``grid_sample`` (bilinear, zero padding, ``align_corners=True``): the output at
    column x is the input at column x - tx."""

    def __init__(self, translation, mode="bilinear", padding_mode="zeros",
                 align_corners=True):
        self.translation = translation
        self.mode, self.padding_mode, self.align_corners = mode, padding_mode, align_corners

    def __call__(self, tensor):
        B, C, H, W = tensor.shape
        dt = tensor.dtype
        t = torch.as_tensor(self.translation).to(dt).reshape(B, 2)
        M = torch.eye(3, dtype=dt).repeat(B, 1, 1)
        M[:, :2, 2] = t

        def norm_pix(h, w):
            tr = torch.tensor([[1.0, 0.0, -1.0], [0.0, 1.0, -1.0], [0.0, 0.0, 1.0]], dtype=dt)
            tr[0, 0] = tr[0, 0] * 2.0 / (1e-14 if w == 1 else w - 1.0)
            tr[1, 1] = tr[1, 1] * 2.0 / (1e-14 if h == 1 else h - 1.0)
            return tr.unsqueeze(0)

        n = norm_pix(H, W)
        theta = torch.inverse(n @ M @ torch.inverse(n))[:, :2, :]
        grid = F.affine_grid(theta, [B, C, H, W], align_corners=self.align_corners)
        return F.grid_sample(tensor, grid, mode=self.mode, padding_mode=self.padding_mode,
                             align_corners=self.align_corners)


def kornia_sampling_matrix(angle: torch.Tensor, center: torch.Tensor, H: int, W: int):
    """[B,2,3] normalised dst->src matrix that kornia feeds to ``affine_grid``."""
    dt = angle.dtype
    B = angle.shape[0]
    pi = torch.tensor(3.14159265358979323846).to(dt)
    ang = angle * pi / 180.0
    cos_a, sin_a = torch.cos(ang), torch.sin(ang)
    rot = torch.stack([cos_a, sin_a, -sin_a, cos_a], dim=-1).view(B, 2, 2)
    eye = torch.eye(3, dtype=dt).expand(B, 3, 3)
    shift = eye.clone(); shift[:, :2, 2] = center
    shift_inv = eye.clone(); shift_inv[:, :2, 2] = -center
    scale = eye.clone()
    rotm = eye.clone(); rotm[:, :2, :2] = rot
    M = shift @ rotm @ scale @ shift_inv
    M3 = eye.clone(); M3[:, :2, :] = M[:, :2, :]

    def norm_pix(h, w):
        tr = torch.tensor([[1.0, 0.0, -1.0], [0.0, 1.0, -1.0], [0.0, 0.0, 1.0]], dtype=dt)
        tr[0, 0] = tr[0, 0] * 2.0 / (1e-14 if w == 1 else w - 1.0)
        tr[1, 1] = tr[1, 1] * 2.0 / (1e-14 if h == 1 else h - 1.0)
        return tr.unsqueeze(0)

    n_src = norm_pix(H, W)
    n_dst = norm_pix(H, W)
    src_pix_from_norm = torch.inverse(n_src)
    dst_norm_from_src_norm = n_dst @ (M3 @ src_pix_from_norm)
    src_norm_from_dst_norm = torch.inverse(dst_norm_from_src_norm)
    return src_norm_from_dst_norm[:, :2, :]


_installed = False


def install():
    """Install the placeholders and put the upstream sources on ``sys.path``."""
    global _installed
    if _installed:
        return
    if not REFERENCE_SRC or not os.path.isdir(os.path.join(REFERENCE_SRC, "pytomography")):
        raise RuntimeError("set PYTOMOGRAPHY_REFERENCE_SRC to the upstream src folder "
                           f"(got {REFERENCE_SRC!r})")
    sys.meta_path.insert(0, _PlaceholderFinder())
    real_version = importlib.metadata.version

    def version(name):
        if name == "pytomography":
            return "3.3.2"
        return real_version(name)

    importlib.metadata.version = version
    sys.path.insert(0, REFERENCE_SRC)
    _installed = True


def import_reference():
    install()
    import pytomography  # noqa: F401
    pytomography.device = torch.device("cpu")
    return pytomography
