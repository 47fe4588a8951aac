"""CPU oracle for the projector hot path.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker (or the timed CPU
baseline); the product library never calls it.

The heavy loops live in ``orc.c`` (built by ``oracle/build.py`` in float64 and
float32); this module restates the host-side logic of the upstream code in
numpy:

* PSF kernel tables: ``get_distance`` (src/pytomography/utils/misc.py:21-38),
  ``SPECTPSFTransform._get_sigma/_compute_kernel_size``
  (src/pytomography/transforms/SPECT/psf.py:170-197) and
  ``get_1D_PSF_layer_gaussian`` (psf.py:62-83);
* the subset split ``indices[i::n]`` (spect_system_matrix.py:58-71);
* ``PoissonLogLikelihood.compute_gradient`` (likelihoods/poisson_log_likelihood.py:16-36);
* the OSEM / BSREM update loop (algorithms/preconditioned_gradient_ascent.py:80-129,
  319-329, 436-474);
* the relative-difference prior gradient (priors/nearest_neighbour.py:44-75,156-183,
  207-220, utils/misc.py:40-57).
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import build as _build

DELTA = 1e-11  # pytomography.delta (src/pytomography/__init__.py:21)

_libs: dict[str, ctypes.CDLL] = {}


def _lib(precision: str) -> ctypes.CDLL:
    if precision not in _libs:
        path = _build.lib_path(precision)
        if not os.path.exists(path):
            _build.build()
        lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        lib.orc_spect_angle.argtypes = [ctypes.c_int, P, P, P, ctypes.c_int, ctypes.c_int,
                                        _real(precision), ctypes.c_double, ctypes.c_char_p,
                                        P, ctypes.c_int, P, ctypes.c_int]
        lib.orc_spect_angle.restype = ctypes.c_int
        lib.orc_spect_plugin.argtypes = [ctypes.c_int, P, P, P, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, _real(precision), ctypes.c_double, P,
                                         ctypes.c_int, P, ctypes.c_int]
        lib.orc_spect_plugin.restype = ctypes.c_int
        R = _real(precision)
        lib.orc_pet_lm.argtypes = [ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int64, P, P, P, P,
                                   P, ctypes.c_int, R, R, R, R, ctypes.c_int]
        lib.orc_pet_lor.argtypes = [ctypes.c_int, P, P, ctypes.c_int64, P, P, P, P, P]
        lib.orc_pet_lor_tof.argtypes = [ctypes.c_int, P, P, ctypes.c_int64, P, P, P, P, P,
                                        ctypes.c_int, R, R, R, R, ctypes.c_int]
        lib.orc_pad_size.argtypes = [ctypes.c_int]
        _libs[precision] = lib
    return _libs[precision]


def _real(precision):
    return ctypes.c_double if precision == "f64" else ctypes.c_float


def _np_dtype(precision):
    return np.float64 if precision == "f64" else np.float32


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def pad_size(n: int) -> int:
    return int(math.ceil((math.sqrt(2) * n - n) / 2))


# ------------------------------------------------------------------ SPECT

def psf_tables(n_pad, dx, dz, radius, a, b, min_sigmas=3.0, two_d=True):
    """Per-plane Gaussian taps for one detector radius: (wr [Lxp,Kr], wz [Lxp,Kz] | None)."""
    if n_pad % 2 == 0:
        d = radius + (n_pad / 2 - np.arange(n_pad) - 0.5) * dx
    else:
        d = radius + ((n_pad - 1) / 2 - np.arange(n_pad)) * dx
    d[d < 0] = 0
    sigma = a * d + b

    def taps(sig_px, K):
        x = np.arange(-(K // 2), K // 2 + 1, dtype=np.float64)[None, :]
        k = np.exp(-x ** 2 / (2 * sig_px[:, None] ** 2 + DELTA))
        return k / k.sum(axis=1, keepdims=True)

    Kr = int(np.ceil(sigma.max() / dx * min_sigmas) * 2 + 1)
    Kz = int(np.ceil(sigma.max() / dz * min_sigmas) * 2 + 1)
    wr = taps(sigma / dx, Kr)
    wz = taps(sigma / dz, Kz) if two_d else None
    return wr, wz


class SpectOracle:
    """Rotate+sum SPECT projector on the CPU (float64 or float32).

    order: obj2obj transform codes in application order, e.g. ``"ap"`` for
    [attenuation, PSF], ``"pa"`` for [PSF, attenuation], ``""`` for none.
    psf: (a, b) of sigma(d) = a*d + b in cm, plus optional min_sigmas / 2D flag.
    """

    def __init__(self, shape, dr, angles, radii=None, mu=None, psf=None, order="",
                 precision="f64", psf_min_sigmas=3.0, psf_2d=True):
        self.shape = tuple(int(s) for s in shape)
        nx, ny, nz = self.shape
        if nx != ny:
            raise ValueError("rotate+sum needs a square transaxial plane")
        self.dr = tuple(float(x) for x in dr)
        self.angles = np.asarray(angles, dtype=np.float64)
        self.radii = np.asarray(radii if radii is not None else np.zeros(len(angles)), np.float64)
        self.precision = precision
        self.dt = _np_dtype(precision)
        self.lib = _lib(precision)
        self.order = order
        self.mu = None if mu is None else np.ascontiguousarray(mu, dtype=self.dt)
        if "a" in order and self.mu is None:
            raise ValueError("attenuation requested without mu")
        self.pad = pad_size(nx)
        self.n_pad = nx + 2 * self.pad
        self.taps = {}
        if "p" in order:
            a, b = psf
            for r in np.unique(self.radii):
                wr, wz = psf_tables(self.n_pad, self.dr[0], self.dr[2], r, a, b,
                                    psf_min_sigmas, psf_2d)
                self.taps[float(r)] = (np.ascontiguousarray(wr, self.dt),
                                       None if wz is None else np.ascontiguousarray(wz, self.dt))

    def _taps(self, i):
        if "p" not in self.order:
            return None, 1, None, 1
        wr, wz = self.taps[float(self.radii[i])]
        return wr, wr.shape[1], wz, (1 if wz is None else wz.shape[1])

    def _call(self, mode, inp, out, i):
        wr, Kr, wz, Kz = self._taps(i)
        rc = self.lib.orc_spect_angle(
            mode, _ptr(inp), _ptr(out), None if self.mu is None else _ptr(self.mu),
            self.shape[0], self.shape[2], self.dt(self.dr[0]), float(self.angles[i]),
            self.order.encode(), None if wr is None else _ptr(wr), Kr,
            None if wz is None else _ptr(wz), Kz)
        if rc != 0:
            raise RuntimeError(f"oracle error {rc}")

    def forward(self, f, angle_idx=None):
        idx = np.arange(len(self.angles)) if angle_idx is None else np.asarray(angle_idx)
        f = np.ascontiguousarray(f, dtype=self.dt)
        out = np.zeros((len(idx), self.shape[1], self.shape[2]), self.dt)
        for j, i in enumerate(idx):
            row = np.zeros((self.shape[1], self.shape[2]), self.dt)
            self._call(0, f, row, int(i))
            out[j] = row
        return out

    def _back(self, mode, g, angle_idx):
        idx = np.arange(len(self.angles)) if angle_idx is None else np.asarray(angle_idx)
        g = np.ascontiguousarray(g, dtype=self.dt)
        out = np.zeros(self.shape, self.dt)
        for j, i in enumerate(idx):
            self._call(mode, np.ascontiguousarray(g[j]), out, int(i))
        return out

    def backward(self, g, angle_idx=None):
        """Reference back-projector: rotate back by +(270 - beta) (SSM:159-201)."""
        return self._back(1, g, angle_idx)

    def adjoint(self, g, angle_idx=None):
        """Exact transpose of :meth:`forward`."""
        return self._back(2, g, angle_idx)


def spect_plugin(which: str, x, dr, beta_deg, mu=None, pad=None, psf=None, radius=0.0,
                 psf_2d=True, precision="f64"):
    """One plugin call on an object already in the detector frame of angle ``beta_deg``
    (orc_spect_plugin): ``which`` = "att" (SPECTAttenuationTransform.forward,
    attenuation.py:72-92) or "psf" (SPECTPSFTransform.forward, psf.py:199-214).
    x: [H, H, Lz] with H = N + 2 pad; pad defaults to the padded frame's."""
    dt = _np_dtype(precision)
    lib = _lib(precision)
    x = np.ascontiguousarray(x, dtype=dt)
    H, _, nz = x.shape
    if which == "att":
        mu = np.ascontiguousarray(mu, dtype=dt)
        n = mu.shape[0]
        pad = pad_size(n) if pad is None else int(pad)
        if n + 2 * pad != H:
            raise ValueError("object frame does not match mu and pad")
        wr = wz = None
        kr = kz = 1
    else:
        n, pad = H, 0
        a, b = psf
        wr, wz = psf_tables(H, dr[0], dr[2], radius, a, b, two_d=psf_2d)
        wr = np.ascontiguousarray(wr, dt)
        wz = None if wz is None else np.ascontiguousarray(wz, dt)
        kr, kz = wr.shape[1], 1 if wz is None else wz.shape[1]
    out = np.empty_like(x)
    rc = lib.orc_spect_plugin(0 if which == "att" else 1, _ptr(x), _ptr(out),
                              None if mu is None else _ptr(mu), n, nz, pad, dt(dr[0]),
                              float(beta_deg), None if wr is None else _ptr(wr), kr,
                              None if wz is None else _ptr(wz), kz)
    if rc != 0:
        raise RuntimeError(f"oracle error {rc}")
    return out


def subsets(n_items: int, n_subsets: int):
    idx = np.arange(n_items)
    return [idx[i::n_subsets] for i in range(n_subsets)]


# --------------------------------------------------------- RDP prior

def rdp_gradient(f, dr, beta, gamma, beta_scale=1.0, fov_scale=None, delta=DELTA):
    """Gradient of the relative-difference prior with Euclidean neighbour weights and
    replicate boundary handling (nearest_neighbour.py:44-75, 156-183, 207-220)."""
    f = np.asarray(f, dtype=np.float64)
    dx, dy, dz = dr
    fp = np.pad(f, 1, mode="edge")
    nx, ny, nz = f.shape
    out = np.zeros_like(f)
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for k in (-1, 0, 1):
                if i == 0 and j == 0 and k == 0:
                    continue
                w = dx / math.sqrt((dx * i) ** 2 + (dy * j) ** 2 + (dz * k) ** 2)
                fs = fp[1 + i:1 + i + nx, 1 + j:1 + j + ny, 1 + k:1 + k + nz]
                d = f - fs
                num = d * (gamma * np.abs(d) + 3 * fs + f + 2 * delta)
                den = (f + fs + gamma * np.abs(d) + delta) ** 2
                out += w * num / den
    out *= beta * beta_scale
    if fov_scale is not None:
        out *= fov_scale
    return out


# ------------------------------------------------ OSEM / BSREM loops

def osem(proj_op, g, n_iters, n_subsets, f0=None, s=None, shape=None, callback=None):
    """OSEM with ``proj_op`` providing forward/backward(angle_idx); returns iterates."""
    A = g.shape[0]
    subs = subsets(A, n_subsets) if n_subsets > 1 else [None]
    f = np.ones(shape) if f0 is None else np.array(f0, dtype=np.float64)
    norm = [proj_op.backward(np.ones((A if k is None else len(k),) + g.shape[1:]), k)
            for k in subs]
    its = []
    for _ in range(n_iters):
        for m, k in enumerate(subs):
            gk = g if k is None else g[k]
            sk = 0 if s is None else (s if k is None else s[k])
            pred = proj_op.forward(f, k) + sk
            grad = proj_op.backward(gk / (pred + DELTA), k) - norm[m]
            f = f + f * (1 / (norm[m] + DELTA)) * grad
            f[f <= 0] = 0
            its.append(f.copy())
    return its, norm


def bsrem(proj_op, g, n_iters, n_subsets, dr, beta, gamma, f0=None, s=None, shape=None,
          relaxation=lambda n: 1.0, floor=1e-4):
    """BSREM with the RDP prior (PGA:80-129, 436-474)."""
    A = g.shape[0]
    subs = subsets(A, n_subsets) if n_subsets > 1 else [None]
    f = np.ones(shape) if f0 is None else np.array(f0, dtype=np.float64)
    norm = [proj_op.backward(np.ones((A if k is None else len(k),) + g.shape[1:]), k)
            for k in subs]
    norm_sum = np.sum(norm, axis=0)
    its = []
    for j in range(n_iters):
        for m, k in enumerate(subs):
            w = 1.0 if k is None else len(k) / A
            vgrad = rdp_gradient(f, dr, beta, gamma, beta_scale=w)
            gk = g if k is None else g[k]
            sk = 0 if s is None else (s if k is None else s[k])
            pred = proj_op.forward(f, k) + sk
            grad = proj_op.backward(gk / (pred + DELTA), k) - norm[m]
            pre = f * (relaxation(j) / (w * norm_sum + DELTA))
            f = f + pre * (grad - vgrad)
            f[f <= floor] = floor
            its.append(f.copy())
    return its, norm


# ------------------------------------------------------------------- PET

class PetLMOracle:
    """Joseph (TOF) listmode projector on the CPU; see ``orc.c`` for the model."""

    def __init__(self, img_shape, voxel_mm, lut, tof=None, precision="f64"):
        self.shape = np.asarray(img_shape, dtype=np.int32)
        self.vox = np.asarray(voxel_mm, dtype=_np_dtype(precision))
        # object origin = (-shape/2 + 0.5) * dr  (petlm_system_matrix.py:46)
        self.origin = ((-self.shape / 2 + 0.5) * np.asarray(voxel_mm)).astype(_np_dtype(precision))
        self.lut = np.ascontiguousarray(lut, dtype=_np_dtype(precision))
        self.tof = tof  # (num_bins, bin_width, sigma, center_offset, n_sigmas)
        self.precision = precision
        self.dt = _np_dtype(precision)
        self.lib = _lib(precision)

    def _args(self):
        if self.tof is None:
            return 0, 1.0, 1.0, 0.0, 3.0, 0
        nb, bw, sig, co, ns = self.tof
        return 1, bw, sig, co, ns, (nb - 1) // 2

    def forward(self, img, ids):
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        img = np.ascontiguousarray(img, dtype=self.dt)
        out = np.zeros(ids.shape[0], self.dt)
        tof, bw, sig, co, ns, shift = self._args()
        R = self.dt
        self.lib.orc_pet_lm(0, _ptr(self.lut), _ptr(ids), ids.shape[1], ids.shape[0], _ptr(img),
                            _ptr(self.shape), _ptr(self.origin), _ptr(self.vox), _ptr(out), tof,
                            R(bw), R(sig), R(co), R(ns), shift)
        return out

    def backward(self, proj, ids):
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        proj = np.ascontiguousarray(proj, dtype=self.dt)
        img = np.zeros(tuple(self.shape), self.dt)
        tof, bw, sig, co, ns, shift = self._args()
        R = self.dt
        self.lib.orc_pet_lm(1, _ptr(self.lut), _ptr(ids), ids.shape[1], ids.shape[0], _ptr(img),
                            _ptr(self.shape), _ptr(self.origin), _ptr(self.vox), _ptr(proj), tof,
                            R(bw), R(sig), R(co), R(ns), shift)
        return img

    def lor_forward(self, img, xs, xe):
        xs = np.ascontiguousarray(xs, self.dt); xe = np.ascontiguousarray(xe, self.dt)
        img = np.ascontiguousarray(img, dtype=self.dt)
        out = np.zeros(xs.shape[0], self.dt)
        self.lib.orc_pet_lor(0, _ptr(xs), _ptr(xe), xs.shape[0], _ptr(img), _ptr(self.shape),
                             _ptr(self.origin), _ptr(self.vox), _ptr(out))
        return out

    def lor_forward_tof(self, img, xs, xe):
        """TOF sinogram projection of explicit LORs: [E, num_bins]."""
        xs = np.ascontiguousarray(xs, self.dt); xe = np.ascontiguousarray(xe, self.dt)
        img = np.ascontiguousarray(img, dtype=self.dt)
        nb = int(self.tof[0])
        out = np.zeros((xs.shape[0], nb), self.dt)
        _, bw, sig, co, ns, shift = self._args()
        R = self.dt
        self.lib.orc_pet_lor_tof(0, _ptr(xs), _ptr(xe), xs.shape[0], _ptr(img), _ptr(self.shape),
                                 _ptr(self.origin), _ptr(self.vox), _ptr(out), nb, R(bw), R(sig),
                                 R(co), R(ns), shift)
        return out

    def lor_backward_tof(self, proj, xs, xe):
        xs = np.ascontiguousarray(xs, self.dt); xe = np.ascontiguousarray(xe, self.dt)
        nb = int(self.tof[0])
        proj = np.ascontiguousarray(proj, self.dt).reshape(xs.shape[0], nb)
        img = np.zeros(tuple(self.shape), self.dt)
        _, bw, sig, co, ns, shift = self._args()
        R = self.dt
        self.lib.orc_pet_lor_tof(1, _ptr(xs), _ptr(xe), xs.shape[0], _ptr(img), _ptr(self.shape),
                                 _ptr(self.origin), _ptr(self.vox), _ptr(proj), nb, R(bw), R(sig),
                                 R(co), R(ns), shift)
        return img

    def lor_backward(self, proj, xs, xe):
        xs = np.ascontiguousarray(xs, self.dt); xe = np.ascontiguousarray(xe, self.dt)
        proj = np.ascontiguousarray(proj, self.dt)
        img = np.zeros(tuple(self.shape), self.dt)
        self.lib.orc_pet_lor(1, _ptr(xs), _ptr(xe), xs.shape[0], _ptr(img), _ptr(self.shape),
                             _ptr(self.origin), _ptr(self.vox), _ptr(proj))
        return img
