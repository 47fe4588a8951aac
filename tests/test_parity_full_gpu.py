"""Full-size parity of the CUDA path against the float64 oracle, per projection and per
OSEM / BSREM iterate, at the sizes of the benchmark configurations.

Tolerance: 1e-5 relative L2 for every compared item (float32 kernels against the float64
restatement in oracle/orc.c, whose SPECT arithmetic is pinned to the reference by the
golden fixtures).  Each test records its largest error, and the terminal summary lists
them per configuration.

Data: the seeded synthetic workloads of pytomography_gb300.synthetic (the reference's
tutorial datasets are not available); the projections are Poisson draws of the CUDA
forward projection of the phantom, and the oracle reconstructs from the same counts.
"""
import numpy as np
import pytest
import torch

import oracle
from conftest import rel_l2, report_parity

TOL = 1e-5
pytestmark = pytest.mark.gpu


class Keep:
    def __init__(self):
        self.its = []

    def run(self, obj, n_iter, n_subset):
        self.its.append(obj.detach().double().cpu().numpy())
        return obj

    def finalize(self, obj):
        pass


def _oracle_for(w, precision="f64"):
    return oracle.SpectOracle(w.shape, w.dr, w.angles, [w.radius] * len(w.angles), mu=w.mu,
                              psf=w.psf, order="ap" if w.psf else "a", precision=precision)


def _oracle_osem_first(o, g, n_subsets, n_first, shape):
    """The oracle's first ``n_first`` OSEM sub-iterations from f = 1 (the update of
    oracle.osem, stopped early; only the subsets used are normalised)."""
    subs = oracle.subsets(g.shape[0], n_subsets)[:n_first]
    f = np.ones(shape)
    its = []
    for k in subs:
        nb = o.backward(np.ones((len(k),) + g.shape[1:]), k)
        pred = o.forward(f, k)
        grad = o.backward(g[k] / (pred + oracle.DELTA), k) - nb
        f = f + f * (1 / (nb + oracle.DELTA)) * grad
        f[f <= 0] = 0
        its.append(f.copy())
    return its


def _check_iterates(name, ours, ref):
    errs = [rel_l2(a, b) for a, b in zip(ours, ref)]
    worst = max(errs)
    report_parity(name, worst)
    assert worst < TOL, (name, int(np.argmax(errs)), worst)


def test_cfg1_osem_every_iterate(cuda):
    """64^3, 64 angles, attenuation, OSEM 4 iterations x 8 subsets: all 32 iterates."""
    from pytomography_gb300 import synthetic
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    w = synthetic.config1()
    H = synthetic.build_system_matrix(w)
    g = synthetic.poisson_projections(H, w).to(cuda)
    o = _oracle_for(w)
    f_true = torch.tensor(w.activity, dtype=torch.float32, device=cuda)
    fwd = H.forward(f_true).cpu().numpy()
    ref = o.forward(w.activity)
    report_parity("cfg1 64^3x64 att: forward, per projection", max(
        rel_l2(fwd[i], ref[i]) for i in range(len(ref))))
    assert rel_l2(fwd, ref) < TOL
    cb = Keep()
    OSEM(PoissonLogLikelihood(H, g))(w.n_iters, w.n_subsets, callback=cb)
    its, _ = oracle.osem(o, g.cpu().numpy().astype(np.float64), w.n_iters, w.n_subsets,
                         shape=w.shape)
    assert len(cb.its) == len(its) == 32
    _check_iterates("cfg1 64^3x64 att: OSEM 4x8, all 32 iterates", cb.its, its)


@pytest.fixture(scope="module")
def cfg2(cuda):
    from pytomography_gb300 import synthetic
    w = synthetic.config2()
    H = synthetic.build_system_matrix(w)
    g = synthetic.poisson_projections(H, w).to(cuda)
    return w, H, g, _oracle_for(w)


def test_cfg2_projections_per_angle(cfg2, cuda):
    """128^3, 120 angles, attenuation + PSF: forward of every angle and both back
    projectors of one subset."""
    w, H, g, o = cfg2
    f = torch.tensor(w.activity, dtype=torch.float32, device=cuda)
    fwd = H.forward(f).cpu().numpy()
    ref = o.forward(w.activity)
    per = [rel_l2(fwd[i], ref[i]) for i in range(len(ref))]
    report_parity("cfg2 128^3x120 att+psf: forward, per projection", max(per))
    assert max(per) < TOL
    H.set_n_subsets(10)
    idx = oracle.subsets(len(w.angles), 10)[3]
    gs = g[torch.as_tensor(idx, device=cuda)].contiguous()
    bwd = H.backward(gs, 3).cpu().numpy()
    e = rel_l2(bwd, o.backward(gs.cpu().numpy().astype(np.float64), idx))
    report_parity("cfg2 128^3x120 att+psf: back projection (reference operator)", e)
    assert e < TOL
    adj = H.backward_adjoint(gs, 3).cpu().numpy()
    e = rel_l2(adj, o.adjoint(gs.cpu().numpy().astype(np.float64), idx))
    report_parity("cfg2 128^3x120 att+psf: back projection (exact adjoint)", e)
    assert e < TOL


def test_cfg2_osem_iterates(cfg2, cuda):
    """OSEM 4 x 10 through the public API: every iterate of the first iteration and every
    later iteration's last iterate against the oracle's run from the same counts."""
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    w, H, g, o = cfg2
    cb = Keep()
    OSEM(PoissonLogLikelihood(H, g))(w.n_iters, w.n_subsets, callback=cb)
    its, _ = oracle.osem(o, g.cpu().numpy().astype(np.float64), w.n_iters, w.n_subsets,
                         shape=w.shape)
    assert len(cb.its) == len(its) == 40
    keep = list(range(10)) + [19, 29, 39]
    _check_iterates("cfg2 128^3x120 att+psf: OSEM 4x10, iterates 1-10, 20, 30, 40",
                    [cb.its[k] for k in keep], [its[k] for k in keep])


def test_cfg4_bsrem_iterates(cfg2, cuda):
    """BSREM with the relative-difference prior (beta 0.3, gamma 2) at the 128^3 / 120-angle
    geometry: the 10 iterates of the first iteration."""
    from pytomography_gb300.algorithms import BSREM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    from pytomography_gb300.priors import RelativeDifferencePrior
    w, H, g, o = cfg2
    cb = Keep()
    BSREM(PoissonLogLikelihood(H, g), prior=RelativeDifferencePrior(beta=0.3, gamma=2))(
        1, w.n_subsets, callback=cb)
    its, _ = oracle.bsrem(o, g.cpu().numpy().astype(np.float64), 1, w.n_subsets, w.dr, 0.3, 2.0,
                          shape=w.shape)
    _check_iterates("cfg4 128^3x120 att+psf: BSREM+RDP, 10 iterates", cb.its, its)


def test_cfg4_batched_gradient(cfg2, cuda):
    """Poisson-NLL gradient of a batch of objects through the autograd Function against
    the oracle's exact adjoint H^T (1 - g / (H f + delta)), one subset."""
    from pytomography_gb300.autograd import poisson_nll
    w, H, g, o = cfg2
    H.set_n_subsets(10)
    idx = oracle.subsets(len(w.angles), 10)[1]
    gs = g[torch.as_tensor(idx, device=cuda)].contiguous()
    rng = np.random.default_rng(4)
    fb = [np.clip(w.activity + rng.uniform(0, 0.5, w.shape), 0, None) for _ in range(2)]
    x = torch.tensor(np.stack(fb), dtype=torch.float32, device=cuda, requires_grad=True)
    poisson_nll(x, H, torch.stack([gs, gs]), subset_idx=1).backward()
    worst = 0.0
    for b in range(2):
        pred = o.forward(fb[b], idx)
        ref = o.adjoint(1 - gs.cpu().numpy() / (pred + oracle.DELTA), idx)
        worst = max(worst, rel_l2(x.grad[b].cpu().numpy(), ref))
    report_parity("cfg4 128^3x120 att+psf: Poisson-NLL gradient (exact adjoint)", worst)
    assert worst < TOL


def test_cfg5_one_reconstruction_per_size_class(cuda):
    """The serving mix: for the first reconstruction of each object size, the batched
    graph-replayed OSEM's first three iterates against the oracle."""
    from pytomography_gb300 import synthetic
    from pytomography_gb300.batched import BatchedOSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    ws = synthetic.config5()
    picked = {}
    for w in ws:
        picked.setdefault(w.shape[0], w)
    ws = [picked[n] for n in sorted(picked)]
    Hs = [synthetic.build_system_matrix(w) for w in ws]
    gs = [synthetic.poisson_projections(H, w).to(cuda) for H, w in zip(Hs, ws)]
    batch = BatchedOSEM([PoissonLogLikelihood(H, g) for H, g in zip(Hs, gs)], n_subsets=10)
    ours = [[] for _ in ws]
    for k in range(3):
        batch.step(k)
        for i, f in enumerate(batch.objects):
            ours[i].append(f.double().cpu().numpy())
    for w, g, mine in zip(ws, gs, ours):
        o = _oracle_for(w)
        its = _oracle_osem_first(o, g.cpu().numpy().astype(np.float64), 10, 3, w.shape)
        _check_iterates(f"cfg5 serving {w.shape[0]}^3x{len(w.angles)}: batched OSEM, "
                        "iterates 1-3", mine, its[:3])


def test_cfg3_pet_listmode_full_image(cuda):
    """PET TOF listmode at the full 200x200x96 image and 600 x 96 crystal scanner with a
    reduced event count (200k): TOF forward and back projection against the float64
    restatement of the Joseph / TOF model (parallelproj is absent, so this pins the
    kernels to the restatement, not to parallelproj)."""
    from pytomography_gb300 import synthetic
    from pytomography_gb300.metadata.PET import PETTOFMeta
    w = synthetic.config3(n_events=200_000)
    H = synthetic.build_pet_system_matrix(w)
    tm = PETTOFMeta(*w.tof)
    o = oracle.PetLMOracle(w.shape, w.voxel_mm, H.proj_meta.scanner_lut.numpy(),
                           tof=(w.tof[0], float(tm.bin_width), float(tm.sigma),
                                float(tm.center_offset), float(tm.n_sigmas)))
    rng = np.random.default_rng(6)
    img = rng.uniform(0.5, 2.0, w.shape)
    f = torch.tensor(img, dtype=torch.float32, device=cuda)
    fwd = H.forward(f).cpu().numpy()
    e = rel_l2(fwd, o.forward(img, w.events))
    report_parity("cfg3 PET 200x200x96 TOF LM: forward (200k events)", e)
    assert e < TOL
    p = rng.uniform(0.5, 2.0, len(w.events))
    bwd = H.backward(torch.tensor(p, dtype=torch.float32, device=cuda)).cpu().numpy()
    e = rel_l2(bwd, o.backward(p, w.events))
    report_parity("cfg3 PET 200x200x96 TOF LM: back projection (200k events)", e)
    assert e < TOL
