"""Plain PyTorch float32 restatement of the reference's per-call SPECT projector.

Test and benchmark infrastructure only: a numerics reference for the CUDA kernels on the
GPU and the "plain per-call GPU projector" that the fused path is timed against.  It
follows the reference's operation sequence one angle at a time, as library calls:

* ``SPECTSystemMatrix.forward`` (src/pytomography/projectors/SPECT/spect_system_matrix.py:
  120-157): pad the object, rotate by ``beta - 270`` (``affine_grid`` / ``grid_sample``,
  bilinear, zeros, ``align_corners=True``, the kornia convention of
  src/pytomography/utils/spatial.py:8-34), apply the obj2obj transforms in order, sum
  along x and crop;
* ``SPECTSystemMatrix.backward`` (spect_system_matrix.py:159-201): broadcast each
  projection along x inside the back-projection box, apply the transforms' backward in
  reverse order, rotate by ``270 - beta``, accumulate and crop;
* ``SPECTAttenuationTransform`` (transforms/SPECT/attenuation.py:11-21, 72-115): the
  attenuation map is padded and rotated by the same angle every call, and
  ``exp(-(rev_cumsum(mu dx) - mu dx / 2))`` multiplies the rotated object;
* ``SPECTPSFTransform`` (transforms/SPECT/psf.py:27-41, 199-231): per-plane taps as
  grouped ``conv1d`` along y, then along z, zero-padded 'same' correlation.

The geometry tables (rotation matrices, PSF taps) are read from a
``pytomography_gb300`` ``SPECTSystemMatrix`` so both sides use identical float32 inputs.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F


class TorchReferenceProjector:
    def __init__(self, H, device=None) -> None:
        from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, \
            SPECTPSFTransform
        self.H = H
        self.device = H.device if device is None else torch.device(device)
        self.N = int(H.object_meta.shape[0])
        self.nz = int(H.object_meta.shape[2])
        self.pad = int(H.object_meta.pad_size)
        self.Lp = self.N + 2 * self.pad
        self.dx = float(H.object_meta.dr[0])
        self.theta_fwd = H._theta_fwd.view(-1, 2, 3).to(self.device)
        self.theta_bwd = H._theta_bwd.view(-1, 2, 3).to(self.device)
        self.transforms = []
        for t in H.obj2obj_transforms:
            if isinstance(t, SPECTAttenuationTransform):
                mu = t.attenuation_map.to(self.device, torch.float32)
                self.transforms.append(("a", self._pad(mu)))
            elif isinstance(t, SPECTPSFTransform):
                taps = {}
                for r, (wr, wz) in t.tables.items():
                    taps[r] = (wr.to(self.device, torch.float32).unsqueeze(1),
                               None if wz is None else
                               wz.to(self.device, torch.float32).unsqueeze(1))
                self.transforms.append(("p", taps))
        self.radii = [float(r) for r in H.proj_meta.radii]
        box = torch.zeros((self.Lp, self.Lp, self.nz), device=self.device)
        box[:, self.pad:self.pad + self.N, :] = 1.0
        self.box = box

    # ------------------------------------------------------------------ pieces
    def _pad(self, x):
        return F.pad(x, [0, 0, self.pad, self.pad, self.pad, self.pad])

    def _rotate(self, x, theta):
        img = x.permute(2, 0, 1).unsqueeze(0)
        grid = F.affine_grid(theta.unsqueeze(0), list(img.shape), align_corners=True)
        r = F.grid_sample(img, grid, mode="bilinear", padding_mode="zeros",
                          align_corners=True)
        return r.squeeze(0).permute(1, 2, 0)

    def _atten(self, mu_pad, theta):
        v = self._rotate(mu_pad, theta) * self.dx
        rev = torch.flip(torch.cumsum(torch.flip(v, (0,)), 0), (0,))
        return torch.exp(-(rev - v / 2))

    def _psf(self, x, taps, radius):
        wr, wz = taps[radius]
        y = F.conv1d(x.permute(2, 0, 1), wr, padding=wr.shape[-1] // 2, groups=self.Lp)
        x = y.permute(1, 2, 0)
        if wz is not None:
            z = F.conv1d(x.permute(1, 0, 2), wz, padding=wz.shape[-1] // 2, groups=self.Lp)
            x = z.permute(1, 0, 2)
        return x

    def _angles(self, subset_idx):
        if subset_idx is None:
            return list(range(self.H.proj_meta.num_projections))
        if isinstance(subset_idx, (list, tuple)):  # explicit angle indices
            return [int(i) for i in subset_idx]
        return [int(i) for i in self.H.subset_indices_array[subset_idx].tolist()]

    # ------------------------------------------------------------------ operators
    def forward(self, f, subset_idx=None):
        fp = self._pad(f.to(self.device, torch.float32))
        out = []
        for a in self._angles(subset_idx):
            th = self.theta_fwd[a]
            v = self._rotate(fp, th)
            for kind, data in self.transforms:
                if kind == "a":
                    v = v * self._atten(data, th)
                else:
                    v = self._psf(v, data, self.radii[a])
            out.append(v.sum(0)[self.pad:self.pad + self.N])
        return torch.stack(out)

    def backward(self, g, subset_idx=None):
        acc = torch.zeros((self.Lp, self.Lp, self.nz), device=self.device)
        for row, a in enumerate(self._angles(subset_idx)):
            p = F.pad(g[row].to(self.device, torch.float32), [0, 0, self.pad, self.pad])
            v = p.unsqueeze(0) * self.box
            for kind, data in reversed(self.transforms):
                if kind == "a":
                    v = v * self._atten(data, self.theta_fwd[a])
                else:
                    v = self._psf(v, data, self.radii[a])
            acc = acc + self._rotate(v, self.theta_bwd[a])
        return acc[self.pad:self.pad + self.N, self.pad:self.pad + self.N]

    def osem_subiteration(self, f, g, s, norm_bp, subset_idx):
        """f + f / (nbp + delta) * (H^T (g / (H f + s + delta)) - nbp), clamped at 0
        (preconditioned_gradient_ascent.py:80-129, poisson_log_likelihood.py:16-36)."""
        delta = 1e-11
        gs = g[self.H.subset_indices_array[subset_idx]] if subset_idx is not None else g
        ss = s[self.H.subset_indices_array[subset_idx]] if (s is not None and
                                                            subset_idx is not None) else s
        pred = self.forward(f, subset_idx)
        if ss is not None:
            pred = pred + ss
        grad = self.backward(gs / (pred + delta), subset_idx) - norm_bp
        f = f + f / (norm_bp + delta) * grad
        return torch.clamp_min(f, 0.0)
