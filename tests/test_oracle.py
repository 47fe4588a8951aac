"""The CPU oracle against the golden fixtures generated from the reference code."""
import numpy as np
import pytest

import oracle
from conftest import golden, order_of, rel_l2


@pytest.mark.parametrize("case", ["spect_even", "spect_odd"])
def test_spect_oracle_matches_reference(case):
    d = golden(case)
    for var in d["variants"]:
        var = str(var)
        o = oracle.SpectOracle(d["shape"], d["dr"], d["angles"], d["radii"], mu=d["mu"],
                               psf=(0.03, 0.11), order=order_of(var), psf_2d="psf1d" not in var)
        fwd = o.forward(d["object"])
        bwd = o.backward(d["proj_in"])
        # float64 oracle vs the reference run in float64: same arithmetic
        assert rel_l2(fwd, d[f"fwd_{var}_f64"]) < 1e-12
        assert rel_l2(bwd, d[f"bwd_{var}_f64"]) < 1e-12
        # vs the reference's float32 run
        assert rel_l2(fwd, d[f"fwd_{var}_f32"]) < 2e-6
        assert rel_l2(bwd, d[f"bwd_{var}_f32"]) < 2e-6
        sub = oracle.subsets(len(d["angles"]), 3)[1]
        assert rel_l2(o.forward(d["object"], sub), d[f"fwd_sub1_{var}_f64"]) < 1e-12
        assert rel_l2(o.backward(d["proj_in"][sub], sub), d[f"bwd_sub1_{var}_f64"]) < 1e-12


def test_oracle_adjoint_is_exact_and_reference_backward_is_not():
    d = golden("spect_even")
    o = oracle.SpectOracle(d["shape"], d["dr"], d["angles"], d["radii"], mu=d["mu"],
                           psf=(0.03, 0.11), order="ap")
    f, g = d["object"], d["proj_in"]
    hf_g = float((o.forward(f) * g).sum())
    assert abs(hf_g - float((f * o.adjoint(g)).sum())) / abs(hf_g) < 1e-13
    assert abs(hf_g - float((f * o.backward(g)).sum())) / abs(hf_g) > 1e-5


def test_psf_tables_match_reference_layers():
    d = golden("spect_even")
    n_pad = int(d["shape"][0]) + 2 * oracle.pad_size(int(d["shape"][0]))
    for r in np.unique(d["radii"]):
        wr, wz = oracle.psf_tables(n_pad, d["dr"][0], d["dr"][2], r, 0.03, 0.11)
        key = f"psf_att+psf_r{float(r):g}"
        assert np.allclose(wr, d[key + "_wr"], atol=1e-7)
        assert np.allclose(wz, d[key + "_wz"], atol=1e-7)


@pytest.mark.parametrize("case", ["osem_small", "osem_additive"])
def test_osem_oracle_matches_reference_iterates(case):
    d = golden(case)
    o = oracle.SpectOracle(d["shape"], d["dr"], d["angles"], d["radii"], mu=d["mu"],
                           psf=(0.03, 0.11), order="ap")
    s = d["additive"] if "additive" in d else None
    its, norm = oracle.osem(o, d["projections"].astype(np.float64), int(d["n_iters"]),
                            int(d["n_subsets"]), shape=tuple(d["shape"]), s=s)
    assert len(its) == len(d["iterates"])
    for a, b in zip(its, d["iterates"]):
        assert rel_l2(a, b) < 2e-6
    assert rel_l2(np.stack(norm), d["norm_bps"]) < 2e-6


def test_bsrem_oracle_matches_reference_iterates():
    d = golden("bsrem_small")
    o = oracle.SpectOracle(d["shape"], d["dr"], d["angles"], d["radii"], mu=d["mu"],
                           psf=(0.03, 0.11), order="ap")
    its, _ = oracle.bsrem(o, d["projections"].astype(np.float64), int(d["n_iters"]),
                          int(d["n_subsets"]), tuple(d["dr"]), float(d["beta"]),
                          float(d["gamma"]), shape=tuple(d["shape"]))
    for a, b in zip(its, d["iterates"]):
        assert rel_l2(a, b) < 2e-6


def test_rdp_oracle_matches_reference():
    d = golden("rdp")
    g = oracle.rdp_gradient(d["object"], d["dr"], float(d["beta"]), float(d["gamma"]),
                            float(d["beta_scale"]))
    assert rel_l2(g, d["grad"]) < 1e-6


def test_pad_sizes():
    assert [oracle.pad_size(n) for n in (15, 16, 64, 96, 128)] == [4, 4, 14, 20, 27]


def test_oracle_plugins_match_reference_plugins():
    """orc_spect_plugin (attenuation and PSF on a detector-frame object) against the
    reference's own SPECTAttenuationTransform / SPECTPSFTransform calls."""
    d = golden("plugins")
    dr = d["dr"]
    for i in (int(v) for v in d["indices"]):
        beta, r = float(d["angles"][i]), float(d["radii"][i])
        xp = d["x_padded"].astype(np.float64)
        xu = d["x_unpadded"].astype(np.float64)
        a = oracle.spect_plugin("att", xp, dr, beta, mu=d["mu"])
        assert rel_l2(a, d[f"att_pad_fwd_{i}_f64"]) < 1e-12
        assert rel_l2(a, d[f"att_pad_fwd_{i}_f32"]) < 1e-6
        a = oracle.spect_plugin("att", xu, dr, beta, mu=d["mu"], pad=0)
        assert rel_l2(a, d[f"att_unpad_fwd_{i}_f32"]) < 1e-6
        p = oracle.spect_plugin("psf", xp, dr, beta, psf=(0.03, 0.11), radius=r)
        assert rel_l2(p, d[f"psf_pad_fwd_{i}_f64"]) < 1e-12
        p = oracle.spect_plugin("psf", xu, dr, beta, psf=(0.03, 0.11), radius=r, psf_2d=False)
        assert rel_l2(p, d[f"psf1d_unpad_fwd_{i}_f32"]) < 1e-6
