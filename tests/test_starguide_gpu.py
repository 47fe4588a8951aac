"""StarGuide system matrix against fixtures made from the reference: forward and back
projection over all detectors and over an angle-group subset, the subset lists and the
subset normalisation, with attenuation, and with attenuation + PSF.  Tolerance 1e-5
relative L2."""
import numpy as np
import pytest
import torch

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _sm(d, with_psf):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTPSFMeta, \
        StarGuideProjMeta
    from pytomography_gb300.projectors.SPECT import StarGuideSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    shape = tuple(int(v) for v in d["shape"])
    om = SPECTObjectMeta([float(v) for v in d["dr"]], shape)
    pm = StarGuideProjMeta((12, 16, shape[2]), torch.tensor(d["angles"], dtype=torch.float32),
                           times=torch.tensor(d["times"], dtype=torch.float32),
                           offsets=torch.tensor(d["offsets"], dtype=torch.float32),
                           radii=[float(r) for r in d["radii"]])
    ts = [SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32),
                                    assume_padded=False)]
    if with_psf:
        ts.append(SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)), assume_padded=False))
    return StarGuideSystemMatrix(om, pm, obj2obj_transforms=ts)


@pytest.mark.parametrize("name,with_psf", [("att", False), ("att_psf", True)])
def test_starguide_matches_reference(name, with_psf, cuda):
    d = golden("starguide")
    H = _sm(d, with_psf)
    f = torch.tensor(d["object"], dtype=torch.float32, device=cuda)
    p = torch.tensor(d["proj"], device=cuda)
    fwd = H.forward(f).cpu().numpy()
    for i in range(12):
        assert rel_l2(fwd[i], d[f"{name}_fwd"][i]) < TOL, i
    assert rel_l2(H.backward(p).cpu().numpy(), d[f"{name}_bwd"]) < TOL
    H.set_n_subsets(2)
    got = np.concatenate([ix.cpu().numpy() for ix in H.subset_indices_array])
    assert np.array_equal(got, d[f"{name}_subsets"])
    assert rel_l2(H.forward(f, 1).cpu().numpy(), d[f"{name}_fwd_s1"]) < TOL
    assert rel_l2(H.backward(H.get_projection_subset(p, 1), 1).cpu().numpy(),
                  d[f"{name}_bwd_s1"]) < TOL
    assert rel_l2(H.compute_normalization_factor(0).cpu().numpy(), d[f"{name}_norm_s0"]) < TOL


def test_starguide_osem_runs_plain_sequence(cuda):
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    d = golden("starguide")
    H = _sm(d, True)
    g = torch.poisson(H.forward(torch.tensor(d["object"], dtype=torch.float32,
                                             device=cuda)).cpu() * 50,
                      generator=torch.Generator().manual_seed(5)).to(cuda)
    alg = OSEM(PoissonLogLikelihood(H, g))
    assert not alg._can_fuse()
    rec = alg(2, 3)
    assert torch.isfinite(rec).all() and float(rec.sum()) > 0
