"""The reference-side binding (pytomography_gb300/reference_binding.py).

CPU: a reference ``SPECTSystemMatrix`` with attenuation and PSF, imported through the
fixture harness, is described field by field: transform order, rotation matrices, the
attenuation map and the PSF taps (the reference's own Conv1d weights, which must equal
this package's host tables bit for bit).  Runs only where the upstream sources are
available (PYTOMOGRAPHY_REFERENCE_SRC); skipped elsewhere.
GPU: the binding's subclass over this package's mirror class (same constructor, same
plugin classes) projects like the golden fixtures, through make_plan and the C ABI.
"""
import os
import sys

import numpy as np
import pytest
import torch

from conftest import GOLDEN, golden, rel_l2


def _reference():
    if not os.environ.get("PYTOMOGRAPHY_REFERENCE_SRC"):
        pytest.skip("upstream sources not available (PYTOMOGRAPHY_REFERENCE_SRC unset)")
    sys.path.insert(0, GOLDEN)
    import refharness
    return refharness.import_reference()


def test_describe_reference_system_matrix():
    _reference()
    from pytomography.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography.projectors.SPECT import SPECTSystemMatrix
    from pytomography.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    from pytomography_gb300 import geometry
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta as MOM
    from pytomography_gb300.metadata.SPECT import SPECTProjMeta as MPM
    from pytomography_gb300.metadata.SPECT import SPECTPSFMeta as MPSF
    from pytomography_gb300.reference_binding import describe
    from pytomography_gb300.transforms.SPECT import SPECTPSFTransform as MPSFT
    d = golden("spect_even")
    shape = tuple(int(s) for s in d["shape"])
    args = ([float(x) for x in d["dr"]], shape)
    pargs = (shape[1:], [float(x) for x in d["dr"][:2]], [float(a) for a in d["angles"]])
    radii = [float(r) for r in d["radii"]]
    mu = torch.tensor(d["mu"], dtype=torch.float32)
    sm = SPECTSystemMatrix([SPECTAttenuationTransform(mu), SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))],
                           [], SPECTObjectMeta(*args), SPECTProjMeta(*pargs, radii=radii))
    f = describe(sm)
    assert f["order"] == "ap" and (f["nx"], f["ny"], f["nz"]) == shape
    Lp = shape[0] + 2 * geometry.compute_pad_size(shape[0])
    ang = torch.tensor(d["angles"], dtype=torch.float32)
    assert np.array_equal(f["theta_fwd"], geometry.rotation_theta(-(270 - ang), Lp).numpy())
    assert np.array_equal(f["theta_bwd"], geometry.rotation_theta(270 - ang, Lp).numpy())
    assert torch.equal(f["mu"], mu)
    mine = MPSFT(MPSF((0.03, 0.11)))
    mine.configure(MOM(*args), MPM(*pargs, radii=radii))
    for gi, r in enumerate(f["psf_radii"]):
        wr, wz = mine.tables[r]
        k = wr.shape[1]
        o = (f["psf_k"] - k) // 2
        assert np.array_equal(f["psf_taps_r"][gi, :, o:o + k], wr.numpy())
        k = wz.shape[1]
        o = (f["psf_k"] - k) // 2
        assert np.array_equal(f["psf_taps_z"][gi, :, o:o + k], wz.numpy())
    assert [f["psf_radii"][g] for g in f["psf_group"]] == radii


@pytest.mark.gpu
def test_bound_subclass_projects_like_the_reference(cuda):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.reference_binding import bind
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    d = golden("spect_even")
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    Bound = bind(SPECTSystemMatrix)
    H = Bound([SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32)),
               SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm)
    f = torch.tensor(d["object"], dtype=torch.float32, device=cuda)
    g = torch.tensor(d["proj_in"], dtype=torch.float32, device=cuda)
    assert rel_l2(H.forward(f).cpu().numpy(), d["fwd_att+psf_f32"]) < 1e-5
    assert rel_l2(H.backward(g).cpu().numpy(), d["bwd_att+psf_f32"]) < 1e-5
    H.set_n_subsets(3)
    assert rel_l2(H.forward(f, 1).cpu().numpy(), d["fwd_sub1_att+psf_f32"]) < 1e-5
