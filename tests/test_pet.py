"""PET listmode path.

CPU: TOF metadata and the scanner LUT against fixtures generated from the reference.
GPU: the TOF / non-TOF Joseph kernels against the float64 oracle restatement
(parallelproj is absent and unpinned, so the Joseph arithmetic itself is pinned only by
the oracle and by model properties), the exact-adjoint dot test, the TOF-sum property,
the sensitivity image and the fused listmode OSEM sub-iteration.  Tolerance 1e-5
relative L2 (float32 kernels vs float64 oracle).
"""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden, rel_l2

TOL = 1e-5

INFO = dict(crystalTransNr=1, crystalTransSpacing=4.0, submoduleTransNr=1,
            submoduleTransSpacing=0.0, moduleTransNr=1, moduleTransSpacing=0.0,
            rsectorTransNr=60, crystalAxialNr=8, crystalAxialSpacing=4.0, submoduleAxialNr=1,
            submoduleAxialSpacing=0.0, moduleAxialNr=1, moduleAxialSpacing=0.0,
            rsectorAxialNr=1, radius=120.0, firstCrystalAxis=1, NrCrystalsPerRing=60, NrRings=8)


def test_tof_meta_matches_reference():
    from pytomography_gb300.metadata.PET import PETTOFMeta
    d = golden("pet_meta")
    for nb, rng_mm, fwhm in ((13, 650.0, 58.5), (12, 600.0, 40.0)):
        m = PETTOFMeta(nb, rng_mm, fwhm)
        got = np.array([float(m.bin_width), float(m.sigma), float(m.center_offset), m.n_sigmas])
        assert np.array_equal(got.astype(np.float32), d[f"tof_{nb}"].astype(np.float32))


def test_scanner_lut_matches_reference():
    from pytomography_gb300.metadata.PET import get_scanner_LUT
    d = golden("pet_meta")
    # torch's float32 sin/cos may differ in the last bit between CPU architectures
    # (the fixtures were made on x86-64): allow 2 ulp at the LUT's 120 mm scale
    np.testing.assert_allclose(get_scanner_LUT(INFO).numpy(), d["lut_small"], rtol=0,
                               atol=2 * np.spacing(np.float32(120.0)))


def _events(lut, n, seed, nb=7, through=None):
    """Random crystal pairs; with `through` (mm), only LORs passing within that transaxial
    distance of the scanner axis (i.e. through the imaged object)."""
    rng = np.random.default_rng(seed)
    i = rng.integers(0, lut.shape[0], 4 * n)
    j = rng.integers(0, lut.shape[0], 4 * n)
    keep = i != j
    if through is not None:
        p0, p1 = lut[i][:, :2], lut[j][:, :2]
        d = p1 - p0
        dist = np.abs(p0[:, 0] * d[:, 1] - p0[:, 1] * d[:, 0]) / np.maximum(
            np.hypot(d[:, 0], d[:, 1]), 1e-9)
        keep &= dist < through
    i, j = i[keep][:n], j[keep][:n]
    t = rng.integers(0, nb, len(i))
    return np.stack([i, j, t], 1).astype(np.int64)


def _setup(tof=True, n_events=3000, seed=0, shape=(40, 36, 16), vox=(2.0, 2.0, 2.0),
           through=None):
    from pytomography_gb300.metadata import ObjectMeta
    from pytomography_gb300.metadata.PET import PETLMProjMeta, PETTOFMeta, get_scanner_LUT
    from pytomography_gb300.projectors.PET import PETLMSystemMatrix
    lut = get_scanner_LUT(INFO)
    ev = _events(lut.numpy(), n_events, seed, through=through)
    tof_meta = PETTOFMeta(7, 210.0, 40.0) if tof else None
    pm = PETLMProjMeta(torch.tensor(ev if tof else ev[:, :2]), scanner_LUT=lut, tof_meta=tof_meta)
    om = ObjectMeta(list(vox), shape)
    H = PETLMSystemMatrix(om, pm, compute_sensitivity=False)
    tofp = None
    if tof:
        tofp = (7, float(tof_meta.bin_width), float(tof_meta.sigma),
                float(tof_meta.center_offset), float(tof_meta.n_sigmas))
    o = oracle.PetLMOracle(shape, vox, lut.numpy(), tof=tofp)
    img = np.random.default_rng(seed + 1).random(shape)
    return H, o, ev if tof else ev[:, :2], img


@pytest.mark.gpu
@pytest.mark.parametrize("tof", [True, False])
def test_pet_forward_backward_vs_oracle(tof, cuda):
    H, o, ev, img = _setup(tof)
    f = torch.tensor(img, dtype=torch.float32, device=cuda)
    fwd = H.forward(f).cpu().numpy()
    ref = o.forward(img, ev)
    assert rel_l2(fwd, ref) < TOL
    p = np.random.default_rng(5).random(len(ev))
    bwd = H.backward(torch.tensor(p, dtype=torch.float32, device=cuda)).cpu().numpy()
    assert rel_l2(bwd, o.backward(p, ev)) < TOL
    H.set_n_subsets(4)
    sub = H.subset_indices_array[2].numpy()
    assert rel_l2(H.forward(f, 2).cpu().numpy(), ref[sub]) < TOL
    b2 = H.backward(torch.tensor(p[sub], dtype=torch.float32, device=cuda), 2).cpu().numpy()
    assert rel_l2(b2, o.backward(p[sub], ev[sub])) < TOL


@pytest.mark.gpu
def test_pet_backward_odd_image_and_alignment(cuda):
    """An image whose voxel count is not a multiple of 4 (the 16-byte vector atomics stop
    at the image end), and the C entry point's 16-byte alignment check of the image."""
    from pytomography_gb300 import _lib
    shape = (15, 13, 7)
    H, o, ev, img = _setup(True, shape=shape, vox=(8.0, 8.0, 8.0))
    p = np.random.default_rng(5).random(len(ev))
    pt = torch.tensor(p, dtype=torch.float32, device=cuda)
    bwd = H.backward(pt).cpu().numpy()
    ref = o.backward(p, ev)
    assert np.abs(ref).sum() > 0
    assert rel_l2(bwd, ref) < TOL
    buf = torch.zeros(int(np.prod(shape)) + 4, device=cuda)
    rc = H._lib.gb_pet_backward(H._plan, _lib.ptr(pt), buf.data_ptr() + 4, -1,
                                _lib.stream_handle(cuda))
    assert rc != 0  # rejected on the host: nothing launched
    assert float(buf.abs().sum()) == 0.0


@pytest.mark.gpu
def test_pet_adjoint_dot(cuda):
    H, o, ev, img = _setup(True, n_events=5000, seed=3)
    f = torch.tensor(img, dtype=torch.float64, device=cuda)
    p = torch.tensor(np.random.default_rng(9).random(len(ev)), device=cuda)
    a = float((H.forward(f.float()).double() * p).sum())
    b = float((f * H.backward(p.float()).double()).sum())
    assert abs(a - b) / abs(a) < 1e-5


@pytest.mark.gpu
def test_tof_bins_sum_to_non_tof(cuda):
    """Summed over every TOF bin that covers the LOR, the TOF projection equals the
    non-TOF projection (the Gaussian bin integrals sum to one inside the window)."""
    from pytomography_gb300.metadata import ObjectMeta
    from pytomography_gb300.metadata.PET import PETLMProjMeta, PETTOFMeta, get_scanner_LUT
    from pytomography_gb300.projectors.PET import PETLMSystemMatrix
    lut = get_scanner_LUT(INFO)
    nb = 61
    base = _events(lut.numpy(), 40, 11)[:, :2]
    ev = np.concatenate([np.concatenate([base, np.full((len(base), 1), b)], 1)
                         for b in range(nb)])
    tm = PETTOFMeta(nb, 61 * 10.0, 20.0)
    om = ObjectMeta([2.0] * 3, (40, 36, 16))
    Ht = PETLMSystemMatrix(om, PETLMProjMeta(torch.tensor(ev), scanner_LUT=lut, tof_meta=tm),
                           compute_sensitivity=False)
    Hn = PETLMSystemMatrix(om, PETLMProjMeta(torch.tensor(base), scanner_LUT=lut),
                           compute_sensitivity=False)
    f = torch.rand((40, 36, 16), device=cuda)
    tof = Ht.forward(f).view(nb, len(base)).sum(0)
    non = Hn.forward(f)
    assert rel_l2(tof.cpu().numpy(), non.cpu().numpy()) < 1e-3


@pytest.mark.gpu
def test_axis_aligned_lor_is_column_sum(cuda):
    """An LOR along x through voxel centres integrates the column times the voxel size."""
    from pytomography_gb300.metadata import ObjectMeta
    from pytomography_gb300.metadata.PET import PETLMProjMeta
    from pytomography_gb300.projectors.PET import PETLMSystemMatrix
    shape, vox = (20, 10, 6), (2.0, 2.0, 2.0)
    origin = (-np.array(shape) / 2 + 0.5) * np.array(vox)
    y, z = origin[1] + 3 * vox[1], origin[2] + 2 * vox[2]
    lut = torch.tensor([[-100.0, y, z], [100.0, y, z]])
    H = PETLMSystemMatrix(ObjectMeta(list(vox), shape),
                          PETLMProjMeta(torch.tensor([[0, 1]]), scanner_LUT=lut),
                          compute_sensitivity=False)
    f = torch.rand(shape, device=cuda)
    got = float(H.forward(f)[0])
    want = float(f[:, 3, 2].sum()) * vox[0]
    assert abs(got - want) / want < 1e-6


@pytest.mark.gpu
def test_sensitivity_all_pairs_vs_oracle(cuda):
    from pytomography_gb300.metadata import ObjectMeta
    from pytomography_gb300.metadata.PET import PETLMProjMeta, get_scanner_LUT
    from pytomography_gb300.projectors.PET import PETLMSystemMatrix
    lut = get_scanner_LUT(INFO)
    shape = (30, 30, 12)
    mu = np.zeros(shape)
    mu[8:22, 8:22, :] = 0.0096
    H = PETLMSystemMatrix(ObjectMeta([2.0] * 3, shape),
                          PETLMProjMeta(torch.tensor([[0, 1]]), scanner_LUT=lut),
                          attenuation_map=torch.tensor(mu, dtype=torch.float32))
    n = lut.shape[0]
    ii, jj = np.triu_indices(n, 1)
    o = oracle.PetLMOracle(shape, [2.0] * 3, lut.numpy())
    xs, xe = lut.numpy()[ii], lut.numpy()[jj]
    att = np.exp(-o.lor_forward(mu, xs, xe))
    ref = o.lor_backward(att + 1e-11, xs, xe)
    ref[ref < 1e-7] = 1e7
    assert rel_l2(H.norm_BP.cpu().numpy(), ref) < TOL


@pytest.mark.gpu
def test_listmode_osem_step_vs_oracle(cuda):
    """One listmode OSEM sub-iteration from the uniform initial image (events through the
    object, sensitivity over every crystal pair) against the float64 oracle; the fused
    and per-call paths agree with each other to float32 summation order."""
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    H, o, ev, img = _setup(True, n_events=20000, seed=7, through=25.0)
    H.norm_BP = H._backward_full()
    H.norm_BP[H.norm_BP < 1e-7] = 1e7
    res = {}
    for fused in (True, False):
        alg = OSEM(PoissonLogLikelihood(H), fused=fused)
        alg(1, 2, n_subset_specific=0)
        res[fused] = alg.object_prediction.cpu().numpy()
    nb = H.norm_BP.cpu().numpy().astype(np.float64)
    f = H._get_object_initial().cpu().numpy().astype(np.float64)
    e = ev[0::2]
    ratio = 1.0 / (o.forward(f, e) + 1e-11)
    nbk = nb * len(e) / len(ev)
    f = f + f * (1 / (nbk + 1e-11)) * (o.backward(ratio, e) - nbk)
    f[f <= 0] = 0
    sens = nb
    mask = (sens > 1e-3 * sens[sens < 1e6].max()) & (sens < 1e6)
    assert mask.mean() > 0.3
    assert rel_l2(res[True][mask], f[mask]) < TOL
    assert rel_l2(res[True], res[False]) < 1e-6


@pytest.mark.gpu
def test_object_initial_and_fov_scale_match_reference(cuda):
    """_get_object_initial and _get_prior_FOV_scale against the reference's own methods
    (petlm_system_matrix.py:59-89; fixture tests/golden/pet_fov.npz) on the same scanner
    and image grid."""
    d = golden("pet_fov")
    H, _, _, _ = _setup(True, n_events=100, shape=tuple(int(s) for s in d["shape"]),
                        vox=tuple(float(v) for v in d["dr"]))
    assert np.array_equal(H._get_object_initial().cpu().numpy(), d["object_initial"])
    assert np.allclose(H._get_prior_FOV_scale().cpu().numpy(), d["fov_scale"], rtol=0,
                       atol=1e-6)
