"""Object-space operators either side of the projectors, against fixtures made from the
reference: GaussianFilter, KEMTransform (with and without top-N selection),
KEMSystemMatrix over a SPECT system matrix; GaussianFilter as the PET resolution model
against the float64 oracle.  Tolerance 1e-5 relative L2."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _om(d):
    from pytomography_gb300.metadata import ObjectMeta
    return ObjectMeta([float(v) for v in d["dr"]], tuple(int(v) for v in d["shape"]))


@pytest.mark.parametrize("fwhm,ns", [(1.2, 3.0), (0.7, 2.0)])
def test_gaussian_filter_matches_reference(fwhm, ns, cuda):
    from pytomography_gb300.transforms.shared import GaussianFilter
    d = golden("kem_filter")
    gf = GaussianFilter(fwhm, n_sigmas=ns)
    gf.configure(_om(d), None)
    out = gf(torch.tensor(d["object"], device=cuda)).cpu().numpy()
    assert rel_l2(out, d[f"gauss_{fwhm}_{ns}"]) < TOL
    b, _ = gf.backward(torch.tensor(d["object"], device=cuda), torch.ones(out.shape))
    assert rel_l2(b.cpu().numpy(), out) < 1e-7


def test_kem_transform_matches_reference(cuda):
    from pytomography_gb300.transforms.shared import KEMTransform
    d = golden("kem_filter")
    s1, s2 = torch.tensor(d["support1"]), torch.tensor(d["support2"])
    kem = KEMTransform([s1, s2], support_kernels_params=[[0.3], [1.0]],
                       distance_kernel_params=[0.6], size=5)
    kem.configure(_om(d), None)
    f = torch.tensor(d["object"], device=cuda)
    assert rel_l2(kem.forward(f).cpu().numpy(), d["kem_fwd"]) < TOL
    assert torch.equal(kem.backward(f), kem.forward(f))
    kem3 = KEMTransform([s1], support_kernels_params=[[0.2]], distance_kernel_params=[0.5],
                        size=3, top_N=10)
    kem3.configure(_om(d), None)
    assert rel_l2(kem3.forward(f).cpu().numpy(), d["kem3_top10_fwd"]) < TOL


def test_kem_system_matrix_over_spect_matches_reference(cuda):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.projectors.shared import KEMSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform
    from pytomography_gb300.transforms.shared import KEMTransform
    d = golden("kem_filter")
    shape, dr = (12, 12, 8), [0.48, 0.48, 0.48]
    angles = [float(a) for a in d["spect_angles"]]
    H = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(d["spect_mu"]))], [],
                          SPECTObjectMeta(dr, shape),
                          SPECTProjMeta(shape[1:], dr[:2], angles, radii=[20.0] * len(angles)))
    kem = KEMTransform([torch.tensor(d["spect_support"])], support_kernels_params=[[0.5]],
                       distance_kernel_params=[1.0], size=3)
    K = KEMSystemMatrix(H, kem)
    a = torch.tensor(d["spect_alpha"], device=cuda)
    p = torch.tensor(d["spect_proj"], device=cuda)
    assert rel_l2(K.forward(a).cpu().numpy(), d["kem_spect_fwd"]) < TOL
    assert rel_l2(K.backward(p).cpu().numpy(), d["kem_spect_bwd"]) < TOL
    K.set_n_subsets(2)
    assert rel_l2(K.compute_normalization_factor(1).cpu().numpy(), d["kem_spect_norm1"]) < TOL
    assert K.get_weighting_subset(1) == 0.5


def _filter_np(img, kernels):
    from scipy.ndimage import correlate1d
    out = np.asarray(img, np.float64)
    for ax, k in enumerate(kernels):
        out = correlate1d(out, np.asarray(k, np.float64), axis=ax, mode="constant", cval=0.0)
    return out


def test_pet_listmode_with_gaussian_resolution_model(cuda):
    """PETLMSystemMatrix(obj2obj_transforms=[GaussianFilter]): forward = H (G f),
    backward = G (H^T g); OSEM then runs the plain sequence."""
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    from pytomography_gb300.metadata import ObjectMeta
    from pytomography_gb300.metadata.PET import PETLMProjMeta, PETTOFMeta, get_scanner_LUT
    from pytomography_gb300.projectors.PET import PETLMSystemMatrix
    from pytomography_gb300.transforms.shared import GaussianFilter
    info = dict(crystalTransNr=1, crystalTransSpacing=4.0, submoduleTransNr=1,
                submoduleTransSpacing=0.0, moduleTransNr=1, moduleTransSpacing=0.0,
                rsectorTransNr=60, crystalAxialNr=8, crystalAxialSpacing=4.0,
                submoduleAxialNr=1, submoduleAxialSpacing=0.0, moduleAxialNr=1,
                moduleAxialSpacing=0.0, rsectorAxialNr=1, radius=120.0,
                firstCrystalAxis=1, NrCrystalsPerRing=60, NrRings=8)
    shape, vox = (40, 40, 8), (4.0, 4.0, 4.0)
    lut = get_scanner_LUT(info)
    rng = np.random.default_rng(21)
    ids = rng.integers(0, lut.shape[0], (20000, 2))
    ids = ids[ids[:, 0] != ids[:, 1]]
    tbin = rng.integers(0, 9, (ids.shape[0], 1))
    ev = torch.tensor(np.concatenate([ids, tbin], 1), dtype=torch.int32)
    tm = PETTOFMeta(9, 270.0, 40.0)
    gf = GaussianFilter(6.0)
    H = PETLMSystemMatrix(ObjectMeta(list(vox), shape), PETLMProjMeta(ev, info, tof_meta=tm),
                          obj2obj_transforms=[gf])
    o = oracle.PetLMOracle(shape, vox, lut.numpy(),
                           tof=(9, float(tm.bin_width), float(tm.sigma), float(tm.center_offset),
                                float(tm.n_sigmas)))
    img = rng.random(shape) + 0.1
    fwd = H.forward(torch.tensor(img, dtype=torch.float32, device=cuda)).cpu().numpy()
    assert rel_l2(fwd, o.forward(_filter_np(img, gf.kernels), ev.numpy())) < TOL
    g = rng.random(ev.shape[0]) + 0.2
    bwd = H.backward(torch.tensor(g, dtype=torch.float32, device=cuda)).cpu().numpy()
    assert rel_l2(bwd, _filter_np(o.backward(g, ev.numpy()), gf.kernels)) < TOL
    alg = OSEM(PoissonLogLikelihood(H))
    assert not alg._can_fuse()
    rec = alg(1, 2)
    assert torch.isfinite(rec).all() and float(rec.sum()) > 0
