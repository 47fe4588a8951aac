"""Multi-bed SPECT: stitching of bed reconstructions (CPU, exact against the reference's
stitched output for the same bed images) and PGAAMultiBedSPECT over three beds on the GPU
(bed by bed and as batched CUDA graphs), against the reference's reconstruction at 1e-5
relative L2."""
import numpy as np
import pytest
import torch

from conftest import golden, rel_l2


def test_stitching_matches_reference():
    from pytomography_gb300.io.SPECT import stitch_multibed
    d = golden("multibed")
    out = stitch_multibed(torch.tensor(d["beds"]), list(d["z_mm"]), float(d["spacing_mm"]))
    assert out.shape == d["stitched"].shape
    assert np.allclose(out.numpy(), d["stitched"], rtol=0, atol=1e-6 * np.abs(d["stitched"]).max())
    w, zs = stitch_multibed(torch.tensor(d["beds"]), list(d["z_mm"]), float(d["spacing_mm"]),
                            return_stitching_weights=True)
    assert list(zs) == [12, 0, 6]  # beds given at 57.6, 0, 28.8 mm with 4.8 mm slices
    # every stitched slice strictly inside the outer beds is covered exactly once
    cover = np.zeros(22)
    for k in range(3):
        cover[zs[k]:zs[k] + 10] += w[k, 0, 0].numpy()
    assert np.all(cover[1:21] == 1)


def _algs(d, cuda, fused=None):
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    shape = tuple(int(v) for v in d["shape"])
    dr = [float(v) for v in d["dr"]]
    angles = [float(a) for a in d["angles"]]
    algs = []
    for b in range(3):
        H = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(d[f"mu{b}"],
                                                                      dtype=torch.float32)),
                               SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [],
                              SPECTObjectMeta(dr, shape),
                              SPECTProjMeta(shape[1:], dr[:2], angles, radii=[20.0] * len(angles)))
        lik = PoissonLogLikelihood(H, torch.tensor(d[f"proj{b}"], device=cuda))
        algs.append(OSEM(lik, fused=fused))
    return algs


@pytest.mark.gpu
@pytest.mark.parametrize("batched,fused", [(True, None), (False, None), (False, False)])
def test_multibed_osem_matches_reference(batched, fused, cuda):
    from pytomography_gb300.algorithms import PGAAMultiBedSPECT
    d = golden("multibed")
    algs = _algs(d, cuda, fused)
    mb = PGAAMultiBedSPECT(list(d["z_mm"]), algs, slice_spacing=float(d["spacing_mm"]),
                           batched=batched)
    out = mb(2, 3).cpu().numpy()
    assert rel_l2(out, d["stitched"]) < 1e-5
    for k, a in enumerate(algs):
        assert rel_l2(a.object_prediction.cpu().numpy(), d["beds"][k]) < 1e-5


@pytest.mark.gpu
def test_multibed_uncertainty_inside_one_bed(cuda):
    """A mask inside the part of the stitched image that only the middle bed supplies has
    the middle bed's own uncertainty."""
    from pytomography_gb300.algorithms import PGAAMultiBedSPECT
    from pytomography_gb300.callbacks import DataStorageCallback
    d = golden("multibed")
    algs = _algs(d, cuda)
    cbs = [DataStorageCallback(a.likelihood, torch.clone(a.object_prediction)) for a in algs]
    mb = PGAAMultiBedSPECT(list(d["z_mm"]), algs, slice_spacing=float(d["spacing_mm"]))
    mb(2, 3, callback=cbs)
    mask = torch.zeros((16, 16, 22), device=cuda)
    mask[5:11, 5:11, 9:13] = 1  # stitched slices 9-12 come from the bed starting at slice 6
    u_mb, pct = mb.compute_uncertainty(mask, cbs, return_pct=True)
    u_bed = algs[2].compute_uncertainty(mask[:, :, 6:16], cbs[2])
    assert abs(u_mb - u_bed) / u_bed < 1e-6 and pct > 0
