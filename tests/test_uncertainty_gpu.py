"""Uncertainty of a masked sum of counts (compute_uncertainty over a DataStorageCallback)
against the reference's own values on the same data: OSEM (fused step), OSEM with a
post-reconstruction Gaussian filter, an earlier sub-iteration, and BSREM with the RDP
prior (its second derivative on the GPU).  Reconstructions within 1e-5 relative L2;
uncertainties within 1e-4 relative (float32 sums over every stored sub-iteration)."""
import numpy as np
import pytest
import torch

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def _setup(d, cuda):
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    shape = tuple(int(v) for v in d["shape"])
    dr = [float(v) for v in d["dr"]]
    angles = [float(a) for a in d["angles"]]
    H = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32)),
                           SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [],
                          SPECTObjectMeta(dr, shape),
                          SPECTProjMeta(shape[1:], dr[:2], angles,
                                        radii=[float(d["radius"])] * len(angles)))
    lik = PoissonLogLikelihood(H, torch.tensor(d["projections"], device=cuda))
    return H, lik


@pytest.mark.parametrize("fused", [None, False])
def test_osem_uncertainty_matches_reference(fused, cuda):
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.callbacks import DataStorageCallback
    from pytomography_gb300.transforms.shared import GaussianFilter
    d = golden("uncertainty")
    H, lik = _setup(d, cuda)
    alg = OSEM(lik, fused=fused)
    cb = DataStorageCallback(lik, torch.clone(alg.object_prediction))
    rec = alg(2, 3, callback=cb)
    assert rel_l2(rec.cpu().numpy(), d["osem_recon"]) < 1e-5
    mask = torch.tensor(d["mask"], device=cuda)
    a_abs, a_pct = alg.compute_uncertainty(mask, cb, return_pct=True)
    assert abs(a_abs - d["osem_unc"][0]) / d["osem_unc"][0] < 1e-4
    assert abs(a_pct - d["osem_unc"][1]) / d["osem_unc"][1] < 1e-4
    sub3 = alg.compute_uncertainty(mask, cb, subiteration_number=3)
    assert abs(sub3 - float(d["osem_unc_sub3"])) / float(d["osem_unc_sub3"]) < 1e-4
    gf = GaussianFilter(0.8)
    gf.configure(H.object_meta, H.proj_meta)
    filt = alg.compute_uncertainty(mask.to(torch.float32), cb, post_recon_filter=gf)
    assert abs(filt - float(d["osem_unc_filtered"])) / float(d["osem_unc_filtered"]) < 1e-4


def test_bsrem_uncertainty_matches_reference(cuda):
    from pytomography_gb300.algorithms import BSREM
    from pytomography_gb300.callbacks import DataStorageCallback
    from pytomography_gb300.priors import RelativeDifferencePrior
    d = golden("uncertainty")
    H, lik = _setup(d, cuda)
    alg = BSREM(lik, prior=RelativeDifferencePrior(beta=0.3, gamma=2))
    cb = DataStorageCallback(lik, torch.clone(alg.object_prediction))
    rec = alg(2, 3, callback=cb)
    assert rel_l2(rec.cpu().numpy(), d["bsrem_recon"]) < 1e-5
    mask = torch.tensor(d["mask"], device=cuda)
    a_abs, a_pct = alg.compute_uncertainty(mask, cb, return_pct=True)
    assert abs(a_abs - d["bsrem_unc"][0]) / d["bsrem_unc"][0] < 1e-4
    assert abs(a_pct - d["bsrem_unc"][1]) / d["bsrem_unc"][1] < 1e-4
    sub3 = alg.compute_uncertainty(mask, cb, subiteration_number=3)
    assert abs(sub3 - float(d["bsrem_unc_sub3"])) / float(d["bsrem_unc_sub3"]) < 1e-4


def test_rdp_hessian_vector_matches_finite_difference(cuda):
    """The RDP second derivative applied to x equals the directional derivative of the
    gradient, (grad(f + e x) - grad(f - e x)) / 2e, in float64 arithmetic of the torch
    restatement below."""
    from pytomography_gb300.metadata import ObjectMeta
    from pytomography_gb300.priors import RelativeDifferencePrior
    g = torch.Generator(cuda).manual_seed(3)
    f = torch.rand((9, 8, 7), device=cuda, generator=g) + 0.5
    x = torch.rand((9, 8, 7), device=cuda, generator=g)
    p = RelativeDifferencePrior(beta=0.7, gamma=2)
    p.set_object_meta(ObjectMeta([0.4, 0.5, 0.6], (9, 8, 7)))
    p.set_beta_scale(0.5)
    p.set_object(f)
    hv = p(derivative_order=2)(x).double()

    def grad64(ff):
        fp = torch.nn.functional.pad(ff[None, None], (1, 1, 1, 1, 1, 1), mode="replicate")[0, 0]
        out = torch.zeros_like(ff)
        for i in (-1, 0, 1):
            for j in (-1, 0, 1):
                for k in (-1, 0, 1):
                    if i == j == k == 0:
                        continue
                    fs = fp[1 + i:10 + i, 1 + j:9 + j, 1 + k:8 + k]
                    d = ff - fs
                    num = d * (2 * d.abs() + 3 * fs + ff + 2e-11)
                    den = (ff + fs + 2 * d.abs() + 1e-11) ** 2
                    out += float(p.weight((i, j, k))) * num / den
        return 0.7 * 0.5 * out

    e = 1e-4
    fd = (grad64(f.double() + e * x.double()) - grad64(f.double() - e * x.double())) / (2 * e)
    assert rel_l2(hv.cpu().numpy(), fd.cpu().numpy()) < 1e-4
