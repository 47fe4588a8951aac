"""Autograd through the fused projector: gradient parity with torch autograd through the
reference's undecorated operators (golden fixture), dot-product adjoint test, and central
finite differences (eps 1e-3, 64 random voxels) on the float64 oracle.  Tolerance 1e-5
relative L2 for the gradient (float32 kernels vs float64 reference)."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def _sm(d, cuda):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    return SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32)),
                              SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm)


def test_poisson_nll_gradient_matches_reference_autograd(cuda):
    from pytomography_gb300.autograd import poisson_nll
    d = golden("autograd")
    H = _sm(d, cuda)
    f = torch.tensor(d["object"], dtype=torch.float32, device=cuda, requires_grad=True)
    g = torch.tensor(d["projections"], dtype=torch.float32, device=cuda)
    nll = poisson_nll(f, H, g)
    nll.backward()
    assert abs(float(nll) - float(d["nll"])) / abs(float(d["nll"])) < 1e-5
    assert rel_l2(f.grad.cpu().numpy(), d["grad"]) < 1e-5


def test_gradient_is_adjoint_and_batched(cuda):
    from pytomography_gb300.autograd import project
    d = golden("autograd")
    H = _sm(d, cuda)
    fb = torch.rand((3, *d["object"].shape), device=cuda, requires_grad=True)
    w = torch.rand((3, len(d["angles"]), *d["object"].shape[1:]), device=cuda)
    (project(fb, H) * w).sum().backward()
    for b in range(3):
        want = H.backward_adjoint(w[b].contiguous())
        assert rel_l2(fb.grad[b].cpu().numpy(), want.cpu().numpy()) < 1e-6
    x = fb[0].detach()
    y = w[0]
    a = float((H.forward(x).double() * y.double()).sum())
    b = float((x.double() * H.backward_adjoint(y).double()).sum())
    assert abs(a - b) / abs(a) < 2e-6


def test_finite_differences_on_oracle_and_gpu(cuda):
    """FD of the float64 oracle NLL agrees with its analytic adjoint gradient (1e-6), and
    the GPU gradient agrees with that analytic gradient (1e-5)."""
    from pytomography_gb300.autograd import poisson_nll
    d = golden("autograd")
    o = oracle.SpectOracle(d["shape"], d["dr"], d["angles"], d["radii"], mu=d["mu"],
                           psf=(0.03, 0.11), order="ap")
    f0, g = d["object"], d["projections"]

    def nll(f):
        p = o.forward(f)
        return float((p - g * np.log(p + 1e-11)).sum())

    grad = o.adjoint(1 - g / (o.forward(f0) + 1e-11))
    rng = np.random.default_rng(4)
    idx = [tuple(int(rng.integers(0, s)) for s in f0.shape) for _ in range(64)]
    eps = 1e-3
    fd = []
    for i in idx:
        fp, fm = f0.copy(), f0.copy()
        fp[i] += eps
        fm[i] -= eps
        fd.append((nll(fp) - nll(fm)) / (2 * eps))
    an = np.array([grad[i] for i in idx])
    assert rel_l2(an, np.array(fd)) < 1e-6
    H = _sm(d, cuda)
    f = torch.tensor(f0, dtype=torch.float32, device=cuda, requires_grad=True)
    poisson_nll(f, H, torch.tensor(g, dtype=torch.float32, device=cuda)).backward()
    gg = f.grad.cpu().numpy()
    assert rel_l2(np.array([gg[i] for i in idx]), an) < 1e-5
