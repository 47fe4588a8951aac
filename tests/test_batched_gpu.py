"""Batched forms over uneven reconstructions and over batches of objects.

* streams mode: every reconstruction's iterates equal the single-reconstruction fused
  OSEM bit for bit (same kernels, same work split);
* persistent mode (one launch per phase across all reconstructions, work split by the
  cost model over the whole batch): iterates, projections and back projections equal the
  single-plan results within the 1e-5 relative L2 used by every parity test (the chunks
  of an angle differ, so the order of the partial sums differs);
* the batched autograd path equals the object-by-object one.
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _recons(cuda, seed=9, n=3, sizes=(24, 32), angle_counts=(12, 18)):
    from pytomography_gb300 import synthetic
    ws = synthetic.config5(seed=seed, n_recons=n, sizes=sizes, angle_counts=angle_counts)
    Hs = [synthetic.build_system_matrix(w) for w in ws]
    gs = [synthetic.poisson_projections(H, w).to(cuda) for H, w in zip(Hs, ws)]
    return ws, Hs, gs


def test_streams_mode_matches_single_and_plain(cuda):
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.batched import BatchedOSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    ws, Hs, gs = _recons(cuda)
    batch = BatchedOSEM([PoissonLogLikelihood(H, g) for H, g in zip(Hs, gs)], n_subsets=3,
                        mode="streams")
    out = [o.clone() for o in batch(2)]
    for H, g, o in zip(Hs, gs, out):
        single = OSEM(PoissonLogLikelihood(H, g), fused=True)(2, 3)
        assert torch.equal(single, o)
        plain = OSEM(PoissonLogLikelihood(H, g), fused=False)(2, 3)
        assert rel_l2(o.cpu().numpy(), plain.cpu().numpy()) < TOL


def test_persistent_mode_matches_single(cuda):
    """Uneven sizes (24^3, 32^3, 40^3) and angle counts, plans of different PSF tap buckets
    brought to a common one; graphs replayed."""
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.batched import BatchedOSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    ws, Hs, gs = _recons(cuda, seed=11, n=5, sizes=(24, 32, 40), angle_counts=(12, 18, 30))
    buckets = {H.psf_bucket for H in Hs}
    refs = [OSEM(PoissonLogLikelihood(H, g), fused=True)(2, 3).clone() for H, g in zip(Hs, gs)]
    batch = BatchedOSEM([PoissonLogLikelihood(H, g) for H, g in zip(Hs, gs)], n_subsets=3)
    assert batch.mode == "persistent"
    assert len({H.psf_bucket for H in Hs}) == 1 and max(buckets) == Hs[0].psf_bucket
    out = batch(2)
    for o, r in zip(out, refs):
        assert torch.isfinite(o).all()
        assert rel_l2(o.cpu().numpy(), r.cpu().numpy()) < TOL
    # the per-plan path after the bucket change gives the same reconstruction
    for H, g, r in zip(Hs, gs, refs):
        again = OSEM(PoissonLogLikelihood(H, g), fused=True)(2, 3)
        assert rel_l2(again.cpu().numpy(), r.cpu().numpy()) < TOL


def test_batch_projectors_match_plans(cuda):
    """gb_spect_batch_forward / _backward (reference and exact adjoint) against each plan's
    own projector, for a subset and for all angles (more angles than one group of 16)."""
    from pytomography_gb300.batched import SpectBatch, common_psf_bucket
    ws, Hs, gs = _recons(cuda, seed=13, n=3, sizes=(24, 32), angle_counts=(18, 40))
    common_psf_bucket(Hs)
    for H in Hs:
        H.set_n_subsets(3)
    b = SpectBatch(Hs)
    rng = np.random.default_rng(1)
    fs = [torch.tensor(rng.random(w.shape), dtype=torch.float32, device=cuda) for w in ws]
    for sub in (None, 2):
        proj = b.forward(fs, sub)
        for H, f, p in zip(Hs, fs, proj):
            assert rel_l2(p.cpu().numpy(), H.forward(f, sub).cpu().numpy()) < TOL
        gp = [torch.rand_like(p) for p in proj]
        for adj in (False, True):
            back = b.backward(gp, sub, adjoint=adj)
            for H, g, o in zip(Hs, gp, back):
                ref = (H.backward_adjoint if adj else H.backward)(g, sub)
                assert rel_l2(o.cpu().numpy(), ref.cpu().numpy()) < TOL, (sub, adj)
    # the plans' lists change: the batch refuses to run on stale lists
    Hs[1].set_n_subsets(2)
    with pytest.raises(RuntimeError, match="create it again"):
        b.forward(fs, 1)


def test_batched_autograd_matches_object_by_object(cuda):
    from pytomography_gb300 import synthetic
    from pytomography_gb300.autograd import SPECTProjectFn, poisson_nll, project
    w = synthetic.config2(n=32, n_angles=24)
    H = synthetic.build_system_matrix(w)
    H.set_n_subsets(4)
    g = synthetic.poisson_projections(H, w).to(cuda)
    rng = np.random.default_rng(2)
    x = torch.tensor(rng.uniform(0.2, 2.0, (3, *w.shape)), dtype=torch.float32, device=cuda,
                     requires_grad=True)
    idx = H.subset_indices_array[1]
    gsub = torch.stack([g[idx]] * 3)
    nll = poisson_nll(x, H, gsub, subset_idx=1)
    nll.backward()
    assert x.grad is not None
    assert "_autograd_batches" in H.__dict__  # the batched path ran
    for b in range(3):
        xb = x[b].detach().clone().requires_grad_(True)
        pred = SPECTProjectFn.apply(xb, H, 1)
        (pred - g[idx] * torch.log(pred + 1e-11)).sum().backward()
        assert rel_l2(x.grad[b].cpu().numpy(), xb.grad.cpu().numpy()) < TOL
    p = project(x.detach(), H, 1)
    for b in range(3):
        assert rel_l2(p[b].cpu().numpy(), H.forward(x[b].detach(), 1).cpu().numpy()) < TOL


@pytest.mark.parametrize("n_subsets", [1, 10])
def test_batch_gather_sample_forms(n_subsets, cuda):
    """16^3 plans with 40 angles: a block of the batched gather covers 65 rows (4 z quads
    per row), so 16 angle slots per group exceed the per-block sample table (one subset)
    and 4 slots fit it (ten subsets); both forms against each plan's own back projector."""
    from pytomography_gb300.batched import SpectBatch, common_psf_bucket
    ws, Hs, gs = _recons(cuda, seed=17, n=2, sizes=(16,), angle_counts=(40,))
    common_psf_bucket(Hs)
    for H in Hs:
        H.set_n_subsets(n_subsets)
    b = SpectBatch(Hs)
    sub = None if n_subsets == 1 else 3
    rng = np.random.default_rng(2)
    gp = [torch.tensor(rng.random((H._n_sel(sub), 16, 16)), dtype=torch.float32, device=cuda)
          for H in Hs]
    back = b.backward(gp, sub)
    for H, g, o in zip(Hs, gp, back):
        assert rel_l2(o.cpu().numpy(), H.backward(g, sub).cpu().numpy()) < TOL
