"""PET sinogram path: geometry tables and listmode binning pinned to fixtures made from
the reference (io/PET/shared.py), sinogram projectors (TOF and non-TOF) against the float64
oracle.  Tolerance 1e-5 relative L2 (float32 kernels vs float64 oracle)."""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden, rel_l2

TOL = 1e-5
INFO = dict(crystalTransNr=1, crystalTransSpacing=4.0, submoduleTransNr=1,
            submoduleTransSpacing=0.0, moduleTransNr=1, moduleTransSpacing=0.0,
            rsectorTransNr=60, crystalAxialNr=8, crystalAxialSpacing=4.0,
            submoduleAxialNr=1, submoduleAxialSpacing=0.0, moduleAxialNr=1,
            moduleAxialSpacing=0.0, rsectorAxialNr=1, radius=120.0,
            firstCrystalAxis=1, NrCrystalsPerRing=60, NrRings=8, min_rsector_difference=0)
SHAPE, VOX = (40, 40, 8), (4.0, 4.0, 4.0)


def test_sinogram_geometry_matches_reference():
    from pytomography_gb300.metadata.PET import PETSinogramPolygonProjMeta, \
        sinogram_coordinates, sinogram_to_spatial
    d = golden("pet_sino")
    lor, sidx = sinogram_coordinates(INFO)
    assert np.array_equal(lor.numpy(), d["lor_coordinates"])
    assert np.array_equal(sidx.numpy(), d["sinogram_index"])
    det, ring = sinogram_to_spatial(INFO)
    # float32 trig of the scanner LUT may differ by an ulp between CPU architectures
    np.testing.assert_allclose(det.numpy(), d["detector_coordinates"], rtol=0, atol=3e-5)
    np.testing.assert_allclose(ring.numpy(), d["ring_coordinates"], rtol=0, atol=3e-5)
    pm = PETSinogramPolygonProjMeta(INFO)
    assert pm.shape == [30, 61, 64] and pm.N_angles == 30


def _sino_sm(tof=True, att=False):
    from pytomography_gb300.metadata import ObjectMeta
    from pytomography_gb300.metadata.PET import PETSinogramPolygonProjMeta, PETTOFMeta
    from pytomography_gb300.projectors.PET import PETSinogramSystemMatrix
    tm = PETTOFMeta(9, 270.0, 40.0) if tof else None
    pm = PETSinogramPolygonProjMeta(INFO, tm)
    mu = None
    if att:
        x = (np.arange(SHAPE[0]) - (SHAPE[0] - 1) / 2) * VOX[0]
        X, Y = np.meshgrid(x, x, indexing="ij")
        mu = torch.tensor(np.where(X ** 2 + Y ** 2 < 60.0 ** 2, 0.0096, 0.0)[..., None]
                          * np.ones(SHAPE), dtype=torch.float32)
    return PETSinogramSystemMatrix(ObjectMeta(list(VOX), SHAPE), pm, attenuation_map=mu), tm, mu


def _oracle(sm, tm):
    tof = None
    if tm is not None:
        tof = (tm.num_bins, float(tm.bin_width), float(tm.sigma), float(tm.center_offset),
               float(tm.n_sigmas))
    return oracle.PetLMOracle(SHAPE, VOX, sm.proj_meta.scanner_lut.numpy(), tof=tof)


def _img(seed=3):
    rng = np.random.default_rng(seed)
    return rng.random(SHAPE) + 0.2


@pytest.mark.gpu
@pytest.mark.parametrize("tof", [False, True])
def test_sino_forward_backward_vs_oracle(tof, cuda):
    sm, tm, _ = _sino_sm(tof)
    o = _oracle(sm, tm)
    xs, xe = (t.numpy() for t in sm._get_xyz_sinogram_coordinates())
    img = _img()
    fwd = sm.forward(torch.tensor(img, dtype=torch.float32, device=cuda)).cpu().numpy()
    ref = o.lor_forward_tof(img, xs, xe) if tof else o.lor_forward(img, xs, xe)
    assert rel_l2(fwd.reshape(-1), ref.reshape(-1)) < TOL
    g = np.random.default_rng(4).random(ref.shape) + 0.1
    bwd = sm.backward(torch.tensor(g.reshape(fwd.shape), dtype=torch.float32,
                                   device=cuda)).cpu().numpy()
    refb = o.lor_backward_tof(g, xs, xe) if tof else o.lor_backward(g, xs, xe)
    assert rel_l2(bwd, refb) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("tof", [False, True])
def test_sino_adjoint_and_subsets(tof, cuda):
    sm, tm, _ = _sino_sm(tof)
    f = torch.tensor(_img(5), dtype=torch.float32, device=cuda)
    full = sm.forward(f)
    g = torch.rand(full.shape, device=cuda, generator=torch.Generator(cuda).manual_seed(6))
    lhs = float((full.double() * g.double()).sum())
    rhs = float((f.double() * sm.backward(g).double()).sum())
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    sm.set_n_subsets(4)
    for k in (0, 3):
        sub = sm.forward(f, k)
        idx = sm.subset_indices_array[k]
        assert torch.allclose(sub, full[idx], rtol=1e-6, atol=1e-6)
        assert sm.get_weighting_subset(k) == len(idx) / 30
    gb = sm.backward(g[sm.subset_indices_array[1]], 1)
    o = _oracle(sm, tm)
    xs, xe = (t.numpy() for t in sm._get_xyz_sinogram_coordinates(1))
    gn = g[sm.subset_indices_array[1]].double().cpu().numpy().reshape(xs.shape[0], -1)
    refb = o.lor_backward_tof(gn, xs, xe) if tof else o.lor_backward(gn[:, 0], xs, xe)
    assert rel_l2(gb.cpu().numpy(), refb) < TOL


@pytest.mark.gpu
def test_tof_bins_sum_to_nontof(cuda):
    """With a TOF window wider than the field of view, the bins of a LOR add up to its
    non-TOF projection (up to the Gaussian tails beyond the outer bins)."""
    sm_t, _, _ = _sino_sm(True)
    sm_n, _, _ = _sino_sm(False)
    f = torch.tensor(_img(7), dtype=torch.float32, device=cuda)
    assert rel_l2(sm_t.forward(f).sum(-1).cpu().numpy(), sm_n.forward(f).cpu().numpy()) < 2e-3


@pytest.mark.gpu
def test_attenuation_and_normalization(cuda):
    sm, tm, mu = _sino_sm(True, att=True)
    o = _oracle(sm, None)
    xs, xe = (t.numpy() for t in sm._get_xyz_sinogram_coordinates())
    prob = sm._compute_atteunation_probability_projection(None).cpu().numpy().reshape(-1)
    ref = np.exp(-o.lor_forward(mu.numpy(), xs, xe))
    assert rel_l2(prob, ref) < TOL
    nbp = sm.compute_normalization_factor().cpu().numpy()
    assert rel_l2(nbp, o.lor_backward(ref, xs, xe)) < TOL


@pytest.mark.gpu
def test_listmode_to_sinogram_matches_reference(cuda):
    from pytomography_gb300.io.PET.shared import listmode_to_sinogram
    from pytomography_gb300.metadata.PET import PETTOFMeta
    d = golden("pet_sino")
    ev = torch.tensor(d["events"])
    w = torch.tensor(d["weights"])
    assert np.array_equal(listmode_to_sinogram(ev[:, :2], INFO).cpu().numpy(), d["sino"])
    assert rel_l2(listmode_to_sinogram(ev[:, :2], INFO, weights=w).cpu().numpy(),
                  d["sino_w"]) < 1e-6
    assert rel_l2(listmode_to_sinogram(ev[:, :2], INFO, weights=w,
                                       normalization=True).cpu().numpy(), d["sino_norm"]) < 1e-6
    tof = listmode_to_sinogram(ev, INFO, tof_meta=PETTOFMeta(13, 650.0, 58.5))
    assert np.array_equal(tof.cpu().numpy(), d["sino_tof"])


@pytest.mark.gpu
def test_sinogram_osem_from_listmode_counts(cuda):
    """OSEM on a sinogram binned from listmode events: the sinogram system matrix runs the
    reference's plain sequence (forward, ratio, back projection, update) and its iterates
    match the same loop with the oracle projector."""
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    sm, _, _ = _sino_sm(False)
    f_true = torch.tensor(_img(8), dtype=torch.float32, device=cuda)
    g = torch.poisson(sm.forward(f_true).cpu() * 5, generator=torch.Generator().manual_seed(9))
    rec = OSEM(PoissonLogLikelihood(sm, g.to(cuda)))(2, 3).cpu().numpy()
    o = _oracle(sm, None)

    class Op:
        def __init__(self):
            self.sub = sm.subset_indices_array

        def _x(self, k):
            return [t.numpy() for t in sm._get_xyz_sinogram_coordinates(k)]

        def forward(self, f, k):
            xs, xe = self._x(k)
            n = 30 if k is None else len(self.sub[k])
            return o.lor_forward(f, xs, xe).reshape(n, 61, 64)

        def backward(self, p, k):
            xs, xe = self._x(k)
            return o.lor_backward(np.asarray(p).reshape(-1), xs, xe)

    subs = oracle.subsets(30, 3)
    gn = g.double().numpy()
    f = np.ones(SHAPE)
    op = Op()
    for _ in range(2):
        for m in range(3):
            k = subs[m]
            norm = op.backward(np.ones((len(k), 61, 64)), m)
            pred = op.forward(f, m)
            f = f + f / (norm + oracle.DELTA) * (op.backward(gn[k] / (pred + oracle.DELTA), m)
                                                  - norm)
            f[f <= 0] = 0
    assert rel_l2(rec, f) < 1e-4
