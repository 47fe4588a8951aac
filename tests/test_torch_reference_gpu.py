"""The CUDA projector against a plain PyTorch float32 restatement of the reference's
per-call sequence (tests/torch_reference.py), itself pinned to the golden fixtures made
from the reference.  Tolerance 1e-5 relative L2 per projection / back projection."""
import numpy as np
import pytest
import torch

from conftest import golden, rel_l2
from test_spect_gpu import make_sm, t32
from torch_reference import TorchReferenceProjector

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.mark.parametrize("variant", ["none", "att", "psf", "att+psf", "psf+att", "att+psf1d"])
def test_torch_reference_matches_golden(variant, cuda):
    d = golden("spect_even")
    H = make_sm(d, variant, cuda)
    R = TorchReferenceProjector(H)
    f, g = t32(d["object"], cuda), t32(d["proj_in"], cuda)
    assert rel_l2(R.forward(f).cpu().numpy(), d[f"fwd_{variant}_f32"]) < TOL
    assert rel_l2(R.backward(g).cpu().numpy(), d[f"bwd_{variant}_f32"]) < TOL


def test_cuda_matches_torch_reference_128(cuda):
    from pytomography_gb300 import synthetic
    w = synthetic.config2()
    H = synthetic.build_system_matrix(w)
    H.set_n_subsets(10)
    R = TorchReferenceProjector(H)
    f = torch.tensor(w.activity, dtype=torch.float32, device=cuda)
    for k in (0, 7):
        a = H.forward(f, k)
        b = R.forward(f, k)
        for i in range(a.shape[0]):
            assert rel_l2(a[i].cpu().numpy(), b[i].cpu().numpy()) < TOL, (k, i)
        g = torch.rand(a.shape, device=cuda, generator=torch.Generator(cuda).manual_seed(k))
        assert rel_l2(H.backward(g, k).cpu().numpy(), R.backward(g, k).cpu().numpy()) < TOL


def test_osem_subiteration_matches_torch_reference(cuda):
    from pytomography_gb300 import synthetic
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    w = synthetic.config2()
    H = synthetic.build_system_matrix(w)
    g = synthetic.poisson_projections(H, w).to(cuda)
    lik = PoissonLogLikelihood(H, g)
    lik._set_n_subsets(10)
    R = TorchReferenceProjector(H)
    f0 = torch.ones(w.shape, device=cuda)
    ref = f0
    for k in range(3):
        ref = R.osem_subiteration(ref, g, None, lik._get_normBP(k), k)
    f = f0.clone()
    for k in range(3):
        H.osem_step(f, g, None, lik._get_normBP(k), k)
    assert rel_l2(f.cpu().numpy(), ref.cpu().numpy()) < TOL
