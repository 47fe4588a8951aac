"""The obj2obj plugins called one angle at a time, as the reference's per-angle loop calls
them (projectors/SPECT/spect_system_matrix.py:145-154, 188-198).

Tolerance: 1e-5 relative L2 against the reference's own plugin outputs
(tests/golden/plugins.npz, float32 and float64 runs of SPECTAttenuationTransform and
SPECTPSFTransform) and against the float64 oracle.
"""
import numpy as np
import pytest
import torch

import oracle
from conftest import golden, rel_l2

TOL = 1e-5
pytestmark = pytest.mark.gpu


def _metas(d):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta
    shape = tuple(int(s) for s in d["shape"])
    om = SPECTObjectMeta([float(x) for x in d["dr"]], shape)
    pm = SPECTProjMeta(shape[1:], [float(x) for x in d["dr"][:2]],
                       [float(a) for a in d["angles"]], radii=[float(r) for r in d["radii"]])
    return om, pm


def _plugins(d, padded):
    from pytomography_gb300.metadata.SPECT import SPECTPSFMeta
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    om, pm = _metas(d)
    att = SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32),
                                    assume_padded=padded)
    psf = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)), assume_padded=padded)
    psf1 = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11), kernel_dimensions="1D"),
                             assume_padded=padded)
    for t in (att, psf, psf1):
        t.configure(om, pm)
    return att, psf, psf1


@pytest.mark.parametrize("frame", ["pad", "unpad"])
def test_plugins_match_reference(frame, cuda):
    d = golden("plugins")
    att, psf, psf1 = _plugins(d, frame == "pad")
    x = torch.tensor(d["x_padded" if frame == "pad" else "x_unpadded"], device=cuda)
    for i in (int(v) for v in d["indices"]):
        ai = torch.tensor(i)  # the reference loop passes 0-d index tensors
        got = {"att_fwd": att.forward(x, ai), "att_bwd": att.backward(x, i),
               "psf_fwd": psf.forward(x, ai), "psf_bwd": psf.backward(x, i),
               "psf1d_fwd": psf1.forward(x, ai)}
        for k, v in got.items():
            key = k.replace("_", "_" + frame + "_", 1)
            v = v.cpu().numpy()
            assert rel_l2(v, d[f"{key}_{i}_f32"]) < TOL, (key, i)
            if f"{key}_{i}_f64" in d:
                assert rel_l2(v, d[f"{key}_{i}_f64"]) < TOL, (key, i)
        # against the float64 oracle's restatement of the same plugin
        beta = float(d["angles"][i])
        o = oracle.spect_plugin("att", d["x_padded" if frame == "pad" else "x_unpadded"],
                                d["dr"], beta, mu=d["mu"], pad=None if frame == "pad" else 0)
        assert rel_l2(got["att_fwd"].cpu().numpy(), o) < TOL
    # the attenuation plugin may run in place
    y = x.clone()
    out = att.forward(y, 3)
    assert rel_l2(out.cpu().numpy(), d[f"att_{frame}_fwd_3_f32"]) < TOL


def test_plugin_chain_equals_fused_forward(cuda):
    """pad -> rotate -> attenuation plugin -> PSF plugin -> sum over x, per angle, equals
    the fused projector's projection of that angle."""
    from pytomography_gb300 import geometry
    from pytomography_gb300.metadata.SPECT import SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    d = golden("spect_even")
    om, pm = _metas(d)
    att = SPECTAttenuationTransform(torch.tensor(d["mu"], dtype=torch.float32))
    psf = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))
    H = SPECTSystemMatrix([att, psf], [], om, pm)
    f = torch.tensor(d["object"], dtype=torch.float32, device=cuda)
    fused = H.forward(f).cpu().numpy()
    pad = om.pad_size
    fp = torch.nn.functional.pad(f, [0, 0, pad, pad, pad, pad])
    L = fp.shape[0]
    theta = geometry.rotation_theta(-(270 - pm.angles), L).view(-1, 2, 3).to(cuda)
    img = fp.permute(2, 0, 1).unsqueeze(0)
    for i in range(len(d["angles"])):
        grid = torch.nn.functional.affine_grid(theta[i:i + 1], list(img.shape),
                                               align_corners=True)
        r = torch.nn.functional.grid_sample(img, grid, mode="bilinear", padding_mode="zeros",
                                            align_corners=True)[0].permute(1, 2, 0).contiguous()
        r = psf.forward(att.forward(r, i), i)
        row = r.sum(0)[pad:pad + f.shape[1]].cpu().numpy()
        assert rel_l2(row, fused[i]) < TOL, i


def test_plugin_arguments_are_checked(cuda):
    d = golden("plugins")
    att, psf, _ = _plugins(d, True)
    with pytest.raises(ValueError):
        att.forward(torch.zeros((3, 3, 3), device=cuda), 0)
    with pytest.raises(RuntimeError, match="GPU"):
        psf.forward(torch.zeros(tuple(int(s) for s in torch.tensor(d["x_padded"]).shape)), 0)
