"""Known-answer checks of the PET Joseph / TOF kernels that do not go through the oracle.

parallelproj, which holds the reference's PET arithmetic, is absent, so the kernels are
pinned by the restatement in oracle/orc.c; these cases derive their answers from the
documented model in closed form instead, so the restatement cannot share a bug with them:

* uniform box, oblique LORs that cross the whole box along their principal axis:
  J = value * n_k * vox_k * |d| / |d_k|  (exact);
* a smooth radial blob, LORs at arbitrary angles and offsets: J ~ the analytic line
  integral of the continuous blob (1% : bilinear interpolation on a 2 mm grid);
* a single hot voxel on an axis-aligned LOR, every TOF bin: vox * the Gaussian integrated
  over the bin, (erf((s + bw/2)/(sqrt2 sigma)) - erf((s - bw/2)/(sqrt2 sigma))) / 2 with s
  the signed distance (towards crystal 2) of the voxel from the bin centre, zero beyond
  n_sigmas sigma + bw/2; both LOR directions (the profile mirrors);
* sensitivity over every crystal pair of a small ring: its inner product with an image
  equals the sum of the image's line integrals over all pairs (forward kernel), and the
  device-generated pairs equal an explicit pair list;
* the deterministic back projection: bit-identical on repeated calls, and equal to the
  float-atomic path to rounding.
"""
import math

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _lm(shape, vox, lut, events, tof=None):
    from pytomography_gb300.metadata import ObjectMeta
    from pytomography_gb300.metadata.PET import PETLMProjMeta
    from pytomography_gb300.projectors.PET import PETLMSystemMatrix
    pm = PETLMProjMeta(torch.as_tensor(np.asarray(events)), scanner_LUT=torch.as_tensor(
        np.asarray(lut, np.float32)), tof_meta=tof)
    return PETLMSystemMatrix(ObjectMeta(list(vox), tuple(shape)), pm, compute_sensitivity=False)


def test_uniform_box_oblique_chords(cuda):
    shape, vox = (40, 36, 16), (2.0, 2.5, 3.0)
    half = np.array(shape) * np.array(vox) / 2
    rng = np.random.default_rng(0)
    lut, events, want = [], [], []
    v = 1.75
    for k in range(3):  # principal axis
        for _ in range(20):
            a, b = (k + 1) % 3, (k + 2) % 3
            p0, p1 = np.zeros(3), np.zeros(3)
            p0[k], p1[k] = -400.0, 400.0
            # stay at least one voxel inside the box along the other two axes, with slopes
            # below 1/2 so that k stays the principal axis
            for ax in (a, b):
                m = half[ax] - 1.5 * vox[ax]
                c0 = rng.uniform(-m, m)
                c1 = float(np.clip(c0 + rng.uniform(-0.9, 0.9) * half[k], -m, m))
                # the LOR's value on this axis over the box's extent along k
                slope = (c1 - c0) / (2 * half[k])
                p0[ax] = c0 - slope * (400.0 - half[k])
                p1[ax] = c1 + slope * (400.0 - half[k])
            lut += [p0, p1]
            events.append([len(lut) - 2, len(lut) - 1])
            d = p1 - p0
            want.append(v * shape[k] * vox[k] * np.linalg.norm(d) / abs(d[k]))
    H = _lm(shape, vox, lut, events)
    got = H.forward(torch.full(shape, v, device=cuda)).cpu().numpy()
    assert np.allclose(got, want, rtol=1e-5, atol=0), np.max(np.abs(got / np.array(want) - 1))


def test_smooth_blob_line_integrals(cuda):
    """f = exp(-r^2 / (2 s^2)) transaxially (r from the z axis), uniform in z; a LOR in a
    transaxial plane at distance b from the axis integrates to sqrt(2 pi) s exp(-b^2/2s^2)."""
    shape, vox, s = (96, 96, 5), (2.0, 2.0, 2.0), 12.0
    org = (-np.array(shape) / 2 + 0.5) * np.array(vox)
    X, Y = np.meshgrid(org[0] + vox[0] * np.arange(shape[0]),
                       org[1] + vox[1] * np.arange(shape[1]), indexing="ij")
    f = np.exp(-(X ** 2 + Y ** 2) / (2 * s * s))[:, :, None] * np.ones(shape[2])
    rng = np.random.default_rng(1)
    lut, events, want = [], [], []
    for _ in range(40):
        phi = rng.uniform(0, np.pi)
        b = rng.uniform(-25, 25)
        u = np.array([np.cos(phi), np.sin(phi), 0.0])
        n = np.array([-np.sin(phi), np.cos(phi), 0.0])
        c = b * n
        lut += [c - 400 * u, c + 400 * u]
        events.append([len(lut) - 2, len(lut) - 1])
        want.append(math.sqrt(2 * math.pi) * s * math.exp(-b * b / (2 * s * s)))
    H = _lm(shape, vox, lut, events)
    got = H.forward(torch.tensor(f, dtype=torch.float32, device=cuda)).cpu().numpy()
    assert np.max(np.abs(got - want) / np.max(want)) < 1e-2


@pytest.mark.parametrize("x_mm", [0.0, 24.0, 80.0, -62.0])
def test_tof_profile_of_a_hot_voxel(x_mm, cuda):
    from pytomography_gb300.metadata.PET import PETTOFMeta
    shape, vox = (101, 61, 5), (2.0, 2.0, 2.0)  # odd: voxel centres on the axes
    org = (-np.array(shape) / 2 + 0.5) * np.array(vox)
    f = np.zeros(shape, np.float32)
    ix = int(round((x_mm - org[0]) / vox[0]))
    f[ix, shape[1] // 2, shape[2] // 2] = 1.0
    tm = PETTOFMeta(13, 650.0, 58.5)
    nb, bw, sig, ns = 13, float(tm.bin_width), float(tm.sigma), float(tm.n_sigmas)
    lut = [[300.0, 0.0, 0.0], [-300.0, 0.0, 0.0]]
    events = [[0, 1, k] for k in range(nb)] + [[1, 0, k] for k in range(nb)]
    H = _lm(shape, vox, lut, events, tof=tm)
    got = H.forward(torch.tensor(f, device=cuda)).cpu().numpy()
    want = []
    for sign in (-1.0, 1.0):  # crystal 2 at -x, then at +x
        for k in range(nb):
            t = (k - (nb - 1) // 2) * bw  # bin centre along the LOR (odd bins: no offset)
            sd = sign * x_mm - t
            if abs(sd) > ns * sig + bw / 2:
                want.append(0.0)
                continue
            q = 1.0 / (math.sqrt(2.0) * sig)
            w = 0.5 * (math.erf((sd + bw / 2) * q) - math.erf((sd - bw / 2) * q))
            want.append(vox[0] * w)
    want = np.array(want)
    assert np.max(np.abs(got - want)) < 1e-5 * want.max(), (got, want)
    # the mirrored direction gives the mirrored profile
    assert np.argmax(got[:nb]) == nb - 1 - np.argmax(got[nb:])


def test_sensitivity_small_ring_equals_sum_of_line_integrals(cuda):
    from pytomography_gb300 import _lib
    from pytomography_gb300.metadata.PET import get_scanner_LUT
    info = dict(crystalTransNr=1, crystalTransSpacing=4.0, submoduleTransNr=1,
                submoduleTransSpacing=0.0, moduleTransNr=1, moduleTransSpacing=0.0,
                rsectorTransNr=48, crystalAxialNr=4, crystalAxialSpacing=4.0,
                submoduleAxialNr=1, submoduleAxialSpacing=0.0, moduleAxialNr=1,
                moduleAxialSpacing=0.0, rsectorAxialNr=1, radius=90.0, firstCrystalAxis=1,
                NrCrystalsPerRing=48, NrRings=4)
    lut = get_scanner_LUT(info).numpy()
    n = lut.shape[0]
    ii, jj = np.triu_indices(n, 1)
    pairs = np.stack([ii, jj], 1).astype(np.int64)
    shape = (40, 40, 8)
    H = _lm(shape, (3.0, 3.0, 2.0), lut, pairs)
    rng = np.random.default_rng(2)
    x = torch.tensor(rng.random(shape), dtype=torch.float32, device=cuda)
    sens = torch.empty(shape, device=cuda)
    _lib.check(H._lib.gb_pet_sensitivity(H._plan, None, 0, None, None, 0.0, _lib.ptr(sens),
                                         _lib.stream_handle(cuda)))
    pd = torch.tensor(pairs.astype(np.int32), device=cuda).contiguous()
    sens2 = torch.empty(shape, device=cuda)
    _lib.check(H._lib.gb_pet_sensitivity(H._plan, _lib.ptr(pd), len(pairs), None, None, 0.0,
                                         _lib.ptr(sens2), _lib.stream_handle(cuda)))
    assert rel_l2(sens.cpu().numpy(), sens2.cpu().numpy()) < 1e-6
    lhs = float((sens.double() * x.double()).sum())
    rhs = float(H.forward(x).double().sum())
    assert abs(lhs - rhs) / abs(rhs) < 1e-5


def test_deterministic_back_projection(cuda):
    from pytomography_gb300 import synthetic
    w = synthetic.config3(n_events=300_000, shape=(100, 100, 48), voxel_mm=(4.0, 4.0, 4.0))
    H = synthetic.build_pet_system_matrix(w)
    p = torch.rand(len(w.events), device=cuda) * 3
    ref = H.backward(p)
    H.set_deterministic(True)
    a = H.backward(p)
    b = H.backward(p)
    assert torch.equal(a, b)
    assert rel_l2(a.cpu().numpy(), ref.cpu().numpy()) < 1e-6
    H.set_deterministic(False)
    assert rel_l2(H.backward(p).cpu().numpy(), ref.cpu().numpy()) < 1e-6
