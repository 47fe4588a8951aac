"""Kernel tile tunings and the autotuner: every tile configuration computes the same
projections (within float32 summation-order differences) and matches the oracle at
1e-5 relative L2; invalid tunings are rejected with an error."""
import numpy as np
import pytest
import torch

import oracle
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _geometry(n=96, nz=96, n_angles=30, dr=0.442, radius=22.0):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform
    rng = np.random.default_rng(7)
    x = np.linspace(-1, 1, n)
    X, Y = np.meshgrid(x, x, indexing="ij")
    body = ((X / 0.8) ** 2 + (Y / 0.6) ** 2 <= 1)[..., None] * np.ones((1, 1, nz))
    f = body * (1.0 + rng.random(body.shape))
    mu = body * 0.15
    angles = list(np.linspace(0, 360, n_angles + 1)[:-1])
    om = SPECTObjectMeta([dr] * 3, (n, n, nz))
    pm = SPECTProjMeta((n, nz), [dr] * 2, angles, radii=[radius] * n_angles)
    H = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(mu, dtype=torch.float32)),
                           SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm)
    o = oracle.SpectOracle((n, n, nz), (dr,) * 3, angles, [radius] * n_angles, mu=mu,
                           psf=(0.03, 0.11), order="ap")
    return H, o, f


def test_every_tuning_matches_oracle(cuda):
    H, o, f = _geometry()
    H.set_n_subsets(5)
    idx = H.subset_indices_array[1].cpu().numpy()
    ref_f = o.forward(f, idx)
    g = np.random.default_rng(3).random(ref_f.shape)
    ref_b = o.backward(g, idx)
    ft = torch.tensor(f, dtype=torch.float32, device=cuda)
    gt = torch.tensor(g, dtype=torch.float32, device=cuda)
    default = H.get_tuning()
    seen = 0
    for tpb in (512, 768):
        for zt in (0, 48):
            for items in (1, 2):
                try:
                    H.set_tuning(fwd_tpb=tpb, fwd_zt=zt, fwd_items=items, b1_zt=zt,
                                 b1_items=items)
                except RuntimeError:
                    continue  # tile does not fit this geometry
                seen += 1
                fwd = H.forward(ft, 1).cpu().numpy()
                for a in range(fwd.shape[0]):
                    assert rel_l2(fwd[a], ref_f[a]) < TOL, (tpb, zt, items, a)
                assert rel_l2(H.backward(gt, 1).cpu().numpy(), ref_b) < TOL, (tpb, zt, items)
    assert seen >= 4
    H.set_tuning(**default)
    assert H.get_tuning() == default
    assert H.device_status() == 0


def test_autotune_picks_a_valid_tuning_and_caches(cuda):
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    H, o, f = _geometry(n=64, nz=64, n_angles=20)
    H.set_n_subsets(4)
    ft = torch.tensor(f, dtype=torch.float32, device=cuda)
    before = H.forward(ft, 2)
    t = H.autotune(0)
    assert t["fwd_tpb"] in (512, 768) and t["fwd_items"] in (1, 2)
    assert H.get_tuning() == t
    after = H.forward(ft, 2)
    assert float((after - before).norm() / before.norm()) < 1e-6
    assert H._tuning_key(0) in SPECTSystemMatrix._tuning_cache
    assert H.autotune(0) == t  # cache hit


def test_invalid_tunings_raise(cuda):
    H, _, _ = _geometry(n=32, nz=32, n_angles=8)
    with pytest.raises(RuntimeError):
        H.set_tuning(fwd_tpb=384)
    with pytest.raises(RuntimeError):
        H.set_tuning(fwd_items=3)
    with pytest.raises(RuntimeError):
        H.set_tuning(fwd_zt=5)  # not a multiple of the output block
    with pytest.raises(RuntimeError):
        H.set_tuning(b1_zt=4096)


@pytest.mark.parametrize("n,nz,n_angles", [(128, 128, 24), (96, 96, 30), (64, 64, 20),
                                           (128, 100, 12), (40, 24, 10)])
def test_forward_variant2_matches_oracle_and_variant1(n, nz, n_angles, cuda):
    """The cp.async-ring forward (z blur first) against the oracle per projection and
    against the first variant, for one and two work items per CTA slot."""
    H, o, f = _geometry(n=n, nz=nz, n_angles=n_angles)
    H.set_n_subsets(2)
    idx = H.subset_indices_array[1].cpu().numpy()
    ref = o.forward(f, idx)
    ft = torch.tensor(f, dtype=torch.float32, device=cuda)
    H.set_tuning(fwd_variant=1)
    v1 = H.forward(ft, 1).cpu().numpy()
    for items in (1, 2):
        H.set_tuning(fwd_variant=2, fwd_items=items)
        assert H.get_tuning()["fwd_variant"] == 2
        v2 = H.forward(ft, 1).cpu().numpy()
        for a in range(v2.shape[0]):
            assert rel_l2(v2[a], ref[a]) < TOL, (items, a)
        assert rel_l2(v2, v1) < TOL
        assert np.array_equal(v2, H.forward(ft, 1).cpu().numpy())  # deterministic
    assert H.device_status() == 0


def test_forward_variant2_rejected_where_it_does_not_apply(cuda):
    from pytomography_gb300.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta
    from pytomography_gb300.projectors.SPECT import SPECTSystemMatrix
    from pytomography_gb300.transforms.SPECT import SPECTPSFTransform
    om = SPECTObjectMeta([0.442] * 3, (32, 32, 16))
    pm = SPECTProjMeta((32, 16), [0.442] * 2, [0.0, 90.0], radii=[22.0, 22.0])
    H = SPECTSystemMatrix([SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm)
    with pytest.raises(RuntimeError, match="variant 2"):
        H.set_tuning(fwd_variant=2)  # no attenuation


def test_split_osem_step_bit_identical_eager_and_graph(cuda):
    """The fused OSEM step run as two angle halves on two streams (fork / join by events)
    gives bit-identical iterates to the one-stream step, eagerly and replayed from a CUDA
    graph."""
    H, o, f = _geometry(n=64, nz=64, n_angles=24)
    H.set_n_subsets(2)
    ft = torch.tensor(f, dtype=torch.float32, device=cuda)
    g = H.forward(ft).contiguous()
    nbp = H.compute_normalization_factor(1).contiguous()
    res = {}
    for split in (0, 1):
        H.set_tuning(osem_split=split)
        assert H.get_tuning()["osem_split"] == split
        x = torch.ones_like(ft)
        for _ in range(2):
            H.osem_step(x, g, None, nbp, 1)
        torch.cuda.synchronize()
        res[split] = x.clone()
    assert torch.equal(res[0], res[1])
    # recorded in a graph on a side stream (the split step forks onto the plan's stream)
    x = torch.ones_like(ft)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        H.osem_step(x, g, None, nbp, 1)
    torch.cuda.synchronize()
    x.fill_(1.0)
    gr = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gr, stream=s):
        H.osem_step(x, g, None, nbp, 1)
    x.fill_(1.0)
    for _ in range(2):
        gr.replay()
    torch.cuda.synchronize()
    assert torch.equal(x, res[1])
    assert H.device_status() == 0
