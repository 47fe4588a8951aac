"""SPECT projector parity on the GPU: CUDA path vs golden fixtures and the oracle.

Tolerance: 1e-5 relative L2 per projection / per back-projected object (float32
arithmetic against the reference's float32 outputs and the float64 oracle).
"""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden, order_of, rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


def make_sm(d, variant, cuda, **kw):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    ts = []
    for t in variant.split("+"):
        if t == "att":
            ts.append(SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32)))
        elif t == "psf":
            ts.append(SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11))))
        elif t == "psf1d":
            ts.append(SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11), kernel_dimensions="1D")))
    return SPECTSystemMatrix(ts, [], om, pm, **kw)


def t32(a, cuda):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=cuda)


@pytest.mark.parametrize("case", ["spect_even", "spect_odd"])
def test_forward_backward_match_reference(case, cuda):
    d = golden(case)
    for var in [str(v) for v in d["variants"]]:
        H = make_sm(d, var, cuda)
        f, g = t32(d["object"], cuda), t32(d["proj_in"], cuda)
        fwd = H.forward(f).cpu().numpy()
        bwd = H.backward(g).cpu().numpy()
        assert rel_l2(fwd, d[f"fwd_{var}_f32"]) < TOL, var
        assert rel_l2(bwd, d[f"bwd_{var}_f32"]) < TOL, var
        assert rel_l2(fwd, d[f"fwd_{var}_f64"]) < TOL, var
        assert rel_l2(bwd, d[f"bwd_{var}_f64"]) < TOL, var
        H.set_n_subsets(3)
        sub = H.get_projection_subset(g, 1)
        assert rel_l2(H.forward(f, 1).cpu().numpy(), d[f"fwd_sub1_{var}_f32"]) < TOL, var
        assert rel_l2(H.backward(sub, 1).cpu().numpy(), d[f"bwd_sub1_{var}_f32"]) < TOL, var


@pytest.mark.parametrize("case", ["spect_even", "spect_odd"])
def test_exact_adjoint(case, cuda):
    d = golden(case)
    for var in [str(v) for v in d["variants"]]:
        H = make_sm(d, var, cuda)
        f, g = t32(d["object"], cuda), t32(d["proj_in"], cuda)
        o = oracle.SpectOracle(d["shape"], d["dr"], d["angles"], d["radii"], mu=d["mu"],
                               psf=(0.03, 0.11), order=order_of(var), psf_2d="psf1d" not in var)
        adj = H.backward_adjoint(g)
        assert rel_l2(adj.cpu().numpy(), o.adjoint(d["proj_in"])) < TOL, var
        a = float((H.forward(f).double() * g.double()).sum())
        b = float((f.double() * adj.double()).sum())
        assert abs(a - b) / abs(a) < 2e-6, var


def test_reference_backward_reproduces_reference_adjoint_gap(cuda):
    d = golden("spect_even")
    H = make_sm(d, "att+psf", cuda)
    f, g = t32(d["object"], cuda), t32(d["proj_in"], cuda)
    a = float((H.forward(f).double() * g.double()).sum())
    b = float((f.double() * H.backward(g).double()).sum())
    ref_gap = (float((d["fwd_att+psf_f64"] * d["proj_in"]).sum())
               - float((d["object"] * d["bwd_att+psf_f64"]).sum()))
    assert abs((a - b) - ref_gap) / abs(ref_gap) < 1e-2


def test_exact_taps_and_truncated_taps_agree(cuda):
    """psf_trunc_rel=0 keeps every tap of the reference kernel; the default truncation
    (1e-7 of a plane's largest tap) changes the projection far below the 1e-5 budget."""
    d = golden("spect_even")
    f = t32(d["object"], cuda)
    exact = make_sm(d, "att+psf", cuda, psf_trunc_rel=0.0).forward(f).cpu().numpy()
    trunc = make_sm(d, "att+psf", cuda).forward(f).cpu().numpy()
    assert rel_l2(exact, d["fwd_att+psf_f32"]) < TOL
    assert rel_l2(trunc, exact) < 1e-6


def test_deterministic(cuda):
    d = golden("spect_even")
    H = make_sm(d, "att+psf", cuda)
    f, g = t32(d["object"], cuda), t32(d["proj_in"], cuda)
    assert torch.equal(H.forward(f), H.forward(f))
    assert torch.equal(H.backward(g), H.backward(g))


def _synthetic(n, nz, n_angles, seed, att=True):
    rng = np.random.default_rng(seed)
    f = np.zeros((n, n, nz))
    x = np.linspace(-1, 1, n)
    X, Y = np.meshgrid(x, x, indexing="ij")
    body = (X / 0.8) ** 2 + (Y / 0.6) ** 2 <= 1
    f[body] = 1.0
    f += rng.random(f.shape) * 0.5 * body[..., None]
    mu = np.where(body[..., None], 0.15, 0.0) * np.ones((1, 1, nz))
    angles = np.linspace(0, 360, n_angles + 1)[:-1]
    return f, mu, angles


@pytest.mark.parametrize("n,nz,n_angles,order,radius,dr", [
    (64, 64, 64, "a", 25.0, 0.48),       # the 64^3 / 64-angle attenuation geometry
    (128, 128, 120, "ap", 22.0, 0.442),  # the 128^3 / 120-angle att+PSF geometry (one subset)
    (37, 21, 9, "pa", 18.0, 0.5),        # odd sizes, PSF before attenuation
    (20, 1, 5, "ap", 15.0, 0.6),         # a single slice
    (144, 40, 6, "ap", 35.0, 0.442),     # rows beyond 128: run-time shared-memory strides
    (64, 256, 2, "ap", 22.0, 0.442),     # a z slab wider than a tensor box: 1-D row copies
])
def test_full_size_geometries_vs_oracle(n, nz, n_angles, order, radius, dr, cuda):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    f, mu, angles = _synthetic(n, nz, n_angles, seed=n)
    om = SPECTObjectMeta([dr] * 3, (n, n, nz))
    pm = SPECTProjMeta((n, nz), [dr] * 2, list(angles), radii=[radius] * n_angles)
    ts = []
    for c in order:
        ts.append(SPECTAttenuationTransform(torch.tensor(mu, dtype=torch.float32)) if c == "a"
                  else SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11))))
    H = SPECTSystemMatrix(ts, [], om, pm)
    n_sub = 10 if n_angles >= 100 else 1
    H.set_n_subsets(n_sub)
    sub = 3 if n_sub > 1 else None
    idx = H.subset_indices_array[sub].cpu().numpy() if sub is not None else None
    o = oracle.SpectOracle((n, n, nz), (dr,) * 3, angles, [radius] * n_angles, mu=mu,
                           psf=(0.03, 0.11), order=order)
    ft = torch.tensor(f, dtype=torch.float32, device=cuda)
    fwd = H.forward(ft, sub).cpu().numpy()
    ref = o.forward(f, idx)
    for a in range(fwd.shape[0]):
        assert rel_l2(fwd[a], ref[a]) < TOL, a
    g = np.random.default_rng(1).random(ref.shape) * 3
    bwd = H.backward(torch.tensor(g, dtype=torch.float32, device=cuda), sub).cpu().numpy()
    assert rel_l2(bwd, o.backward(g, idx)) < TOL
    adj = H.backward_adjoint(torch.tensor(g, dtype=torch.float32, device=cuda), sub).cpu().numpy()
    assert rel_l2(adj, o.adjoint(g, idx)) < TOL
    assert H.device_status() == 0


@pytest.mark.parametrize("n_sub", [1, 2])
def test_back_projection_sample_table_and_fallback_vs_oracle(n_sub, cuda):
    """16 x 16 x 16 with 10 angles: a gather block covers 64 rows (4 z quads per row), so
    one subset of 10 angles (640 row-angle pairs) takes the per-thread sample form and two
    subsets of 5 (320 pairs) the shared per-block table; both against the oracle."""
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    n, nz, n_angles, dr, radius = 16, 16, 10, 0.5, 15.0
    f, mu, angles = _synthetic(n, nz, n_angles, seed=7)
    om = SPECTObjectMeta([dr] * 3, (n, n, nz))
    pm = SPECTProjMeta((n, nz), [dr] * 2, list(angles), radii=[radius] * n_angles)
    H = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(mu, dtype=torch.float32)),
                           SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm)
    o = oracle.SpectOracle((n, n, nz), (dr,) * 3, angles, [radius] * n_angles, mu=mu,
                           psf=(0.03, 0.11), order="ap")
    rng = np.random.default_rng(3)
    if n_sub == 1:
        g = rng.random((n_angles, n, nz)) * 3
        bwd = H.backward(torch.tensor(g, dtype=torch.float32, device=cuda)).cpu().numpy()
        assert rel_l2(bwd, o.backward(g, None)) < TOL
        return
    H.set_n_subsets(n_sub)
    for k in range(n_sub):
        idx = H.subset_indices_array[k].cpu().numpy()
        g = rng.random((len(idx), n, nz)) * 3
        bwd = H.backward(torch.tensor(g, dtype=torch.float32, device=cuda), k).cpu().numpy()
        assert rel_l2(bwd, o.backward(g, idx)) < TOL, k


def test_normalization_factors_in_one_call_match_per_subset(cuda):
    d = golden("spect_even")
    H = make_sm(d, "att+psf", cuda)
    H.set_n_subsets(3)
    many = H.compute_normalization_factors()
    assert len(many) == 3
    for k in range(3):
        assert torch.equal(many[k], H.compute_normalization_factor(k)), k


def test_object_initial_on_camera_path_matches_reference(cuda):
    """_get_object_initial with object_initial_based_on_camera_path against the reference's
    own mask (spect_system_matrix.py:38-56, fixture tests/golden/camera_path.npz)."""
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    d = golden("camera_path")
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    H = SPECTSystemMatrix([], [], om, pm, object_initial_based_on_camera_path=True)
    init = H._get_object_initial().cpu().numpy()
    ref = d["object_initial"]
    assert rel_l2(init, ref) < TOL
    assert np.abs(init - ref).max() < 1e-5
