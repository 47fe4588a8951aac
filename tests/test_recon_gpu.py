"""OSEM / BSREM / RDP on the GPU vs the reference's iterates (golden fixtures).

Tolerance: 1e-5 relative L2 per iterate, for both the fused sub-iteration and the
plain per-call path.
"""
import numpy as np
import pytest
import torch

from conftest import golden, rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


def _setup(d, cuda):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    att = SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32))
    psf = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))
    H = SPECTSystemMatrix([att, psf], [], om, pm)
    g = torch.tensor(d["projections"], dtype=torch.float32, device=cuda)
    s = torch.tensor(d["additive"], dtype=torch.float32, device=cuda) if "additive" in d else None
    return H, PoissonLogLikelihood(H, g, additive_term=s)


class Keep:
    def __init__(self):
        self.its = []

    def run(self, obj, n_iter, n_subset):
        self.its.append(obj.detach().cpu().numpy().copy())
        return obj

    def finalize(self, obj):
        pass


@pytest.mark.parametrize("case", ["osem_small", "osem_additive"])
@pytest.mark.parametrize("fused", [True, False])
def test_osem_iterates(case, fused, cuda):
    from pytomography_gb300.algorithms import OSEM
    d = golden(case)
    H, lik = _setup(d, cuda)
    cb = Keep()
    OSEM(lik, fused=fused)(int(d["n_iters"]), int(d["n_subsets"]), callback=cb)
    assert len(cb.its) == len(d["iterates"])
    for k, (a, b) in enumerate(zip(cb.its, d["iterates"])):
        assert rel_l2(a, b) < TOL, (k, rel_l2(a, b))
    assert rel_l2(torch.stack(lik.norm_BPs).cpu().numpy(), d["norm_bps"]) < TOL


@pytest.mark.parametrize("fused", [True, False])
def test_bsrem_iterates(fused, cuda):
    from pytomography_gb300.algorithms import BSREM
    from pytomography_gb300.priors import RelativeDifferencePrior
    d = golden("bsrem_small")
    H, lik = _setup(d, cuda)
    cb = Keep()
    prior = RelativeDifferencePrior(beta=float(d["beta"]), gamma=float(d["gamma"]))
    BSREM(lik, prior=prior, fused=fused)(int(d["n_iters"]), int(d["n_subsets"]), callback=cb)
    for k, (a, b) in enumerate(zip(cb.its, d["iterates"])):
        assert rel_l2(a, b) < TOL, (k, rel_l2(a, b))


def test_rdp_gradient(cuda):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta
    from pytomography_gb300.priors import RelativeDifferencePrior
    d = golden("rdp")
    p = RelativeDifferencePrior(beta=float(d["beta"]), gamma=float(d["gamma"]))
    p.set_object_meta(SPECTObjectMeta([float(x) for x in d["dr"]], tuple(d["object"].shape)))
    p.set_object(torch.tensor(d["object"], dtype=torch.float32, device=cuda))
    p.set_beta_scale(float(d["beta_scale"]))
    assert rel_l2(p(derivative_order=1).cpu().numpy(), d["grad"]) < TOL
    assert abs(p(derivative_order=0) - float(d["value"])) / abs(float(d["value"])) < 1e-5


def test_fused_osem_predicted_projections(cuda):
    from pytomography_gb300.algorithms import OSEM
    d = golden("osem_additive")
    H, lik = _setup(d, cuda)
    alg = OSEM(lik)
    alg(1, int(d["n_subsets"]))
    last = int(d["n_subsets"]) - 1
    # projections_predicted after the last sub-iteration equals H_m f_prev + s_m
    assert lik.projections_predicted.shape[0] == H._n_sel(last)
