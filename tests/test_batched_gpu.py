"""Batched OSEM over uneven reconstructions: every reconstruction's iterates equal the
single-reconstruction fused OSEM (same kernels), and the per-call plain path within the
1e-5 relative L2 used by every parity test."""
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_batched_matches_single_and_plain(cuda):
    from pytomography_gb300 import synthetic
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.batched import BatchedOSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    ws = synthetic.config5(seed=9, n_recons=3, sizes=(24, 32), angle_counts=(12, 18))
    Hs = [synthetic.build_system_matrix(w) for w in ws]
    gs = [synthetic.poisson_projections(H, w).to(cuda) for H, w in zip(Hs, ws)]
    batch = BatchedOSEM([PoissonLogLikelihood(H, g) for H, g in zip(Hs, gs)], n_subsets=3)
    out = [o.clone() for o in batch(2)]
    for H, g, o in zip(Hs, gs, out):
        single = OSEM(PoissonLogLikelihood(H, g), fused=True)(2, 3)
        assert torch.equal(single, o)
        plain = OSEM(PoissonLogLikelihood(H, g), fused=False)(2, 3)
        assert rel_l2(o.cpu().numpy(), plain.cpu().numpy()) < 1e-5
