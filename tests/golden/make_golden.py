"""Generate the golden fixtures under ``tests/golden/`` from the upstream code.

Run in a container that holds the upstream PyTomography sources, with
``PYTOMOGRAPHY_REFERENCE_SRC`` naming their ``src`` folder::

    python tests/golden/make_golden.py            # writes every tests/golden/*.npz
    python tests/golden/make_golden.py plugins    # writes only the named cases

Every output in the fixtures is produced by the upstream implementation itself
(``SPECTSystemMatrix.forward/backward``, ``SPECTAttenuationTransform``,
``SPECTPSFTransform``, ``PoissonLogLikelihood``, ``OSEM``, ``BSREM``,
``RelativeDifferencePrior``, ``PETTOFMeta``, ``get_scanner_LUT``) imported
through ``refharness``; only kornia's ``rotate`` is a restatement (see
``refharness``).  Inputs are seeded and stored beside the outputs, so the tests
never regenerate them.  Each SPECT case is run twice: in float32 (the
reference's working precision) and in float64 (``pytomography.set_dtype``),
which pins the float64 oracle.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refharness  # noqa: E402

pt = refharness.import_reference()
from pytomography.metadata.SPECT import SPECTObjectMeta, SPECTProjMeta, SPECTPSFMeta  # noqa: E402
from pytomography.projectors.SPECT import SPECTSystemMatrix  # noqa: E402
from pytomography.transforms.SPECT import SPECTAttenuationTransform, SPECTPSFTransform  # noqa: E402
from pytomography.likelihoods import PoissonLogLikelihood  # noqa: E402
from pytomography.algorithms import OSEM, BSREM  # noqa: E402
from pytomography.priors import RelativeDifferencePrior  # noqa: E402
from pytomography.metadata.PET import PETTOFMeta  # noqa: E402
from pytomography.io.PET import shared as pet_shared  # noqa: E402
from pytomography.utils import compute_pad_size  # noqa: E402


def set_precision(dt):
    pt.set_dtype(dt)


def ellipsoid_phantom(shape, dr, seed, n_ell=3):
    """Small seeded phantom: background cylinder plus hot ellipsoids."""
    g = np.random.default_rng(seed)
    nx, ny, nz = shape
    x = (np.arange(nx) - (nx - 1) / 2) * dr[0]
    y = (np.arange(ny) - (ny - 1) / 2) * dr[1]
    z = (np.arange(nz) - (nz - 1) / 2) * dr[2]
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    rx, ry = 0.42 * nx * dr[0], 0.34 * ny * dr[1]
    body = (X / rx) ** 2 + (Y / ry) ** 2 <= 1
    f = 0.5 * body.astype(np.float64)
    for _ in range(n_ell):
        c = g.uniform(-0.5, 0.5, 3) * np.array([rx, ry, nz * dr[2] * 0.6])
        a = g.uniform(0.15, 0.3, 3) * np.array([rx, ry, nz * dr[2]])
        m = ((X - c[0]) / a[0]) ** 2 + ((Y - c[1]) / a[1]) ** 2 + ((Z - c[2]) / a[2]) ** 2 <= 1
        f[m] = g.uniform(1, 10)
    mu = np.where(body, 0.15, 0.0)
    lung = ((X + 0.35 * rx) / (0.25 * rx)) ** 2 + (Y / (0.4 * ry)) ** 2 <= 1
    mu = np.where(lung, 0.04, mu)
    return f, mu


def spect_case(name, shape, dr, angles, radii, variants, seed, out):
    rng = np.random.default_rng(seed)
    f_np, mu_np = ellipsoid_phantom(shape, dr, seed)
    f_np = f_np + 0.1 * rng.random(shape)
    g_np = rng.random((len(angles), shape[1], shape[2])) * 5
    rec = {"shape": np.array(shape), "dr": np.array(dr), "angles": np.array(angles),
           "radii": np.array(radii), "object": f_np, "mu": mu_np, "proj_in": g_np}
    for prec, dt in (("f32", torch.float32), ("f64", torch.float64)):
        set_precision(dt)
        for var in variants:
            om = SPECTObjectMeta(list(dr), tuple(shape))
            pm = SPECTProjMeta((shape[1], shape[2]), list(dr[:2]), list(angles), radii=list(radii))
            ts = []
            for t in var.split("+"):
                if t == "att":
                    ts.append(SPECTAttenuationTransform(torch.tensor(mu_np, dtype=dt)))
                elif t == "psf":
                    ts.append(SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11))))
                elif t == "psf1d":
                    ts.append(SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11), kernel_dimensions="1D")))
            H = SPECTSystemMatrix(ts, [], om, pm)
            f = torch.tensor(f_np, dtype=dt)
            g = torch.tensor(g_np, dtype=dt)
            rec[f"fwd_{var}_{prec}"] = H.forward(f).numpy()
            rec[f"bwd_{var}_{prec}"] = H.backward(g).numpy()
            H.set_n_subsets(3)
            rec[f"fwd_sub1_{var}_{prec}"] = H.forward(f, 1).numpy()
            rec[f"bwd_sub1_{var}_{prec}"] = H.backward(H.get_projection_subset(g, 1), 1).numpy()
            if prec == "f32":
                for t in ts:
                    if isinstance(t, SPECTPSFTransform):
                        for r, layer in t.layers.items():
                            key = f"psf_{var}_r{float(r):g}"
                            rec[key + "_wr"] = layer.layer_r.weight.detach().numpy()[:, 0, :]
                            if layer.layer_z is not None:
                                rec[key + "_wz"] = layer.layer_z.weight.detach().numpy()[:, 0, :]
    set_precision(torch.float32)
    rec["variants"] = np.array(variants)
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **rec)
    print("wrote", name)


def osem_case(name, shape, dr, angles, radius, n_iters, n_subsets, seed, out,
              bsrem=False, additive=False):
    f_true, mu_np = ellipsoid_phantom(shape, dr, seed, n_ell=2)
    rec = {"shape": np.array(shape), "dr": np.array(dr), "angles": np.array(angles),
           "radii": np.full(len(angles), radius), "object_true": f_true, "mu": mu_np,
           "n_iters": n_iters, "n_subsets": n_subsets}
    set_precision(torch.float32)
    om = SPECTObjectMeta(list(dr), tuple(shape))
    pm = SPECTProjMeta((shape[1], shape[2]), list(dr[:2]), list(angles), radii=[radius] * len(angles))
    att = SPECTAttenuationTransform(torch.tensor(mu_np, dtype=torch.float32))
    psf = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))
    H = SPECTSystemMatrix([att, psf], [], om, pm)
    gen = torch.Generator().manual_seed(seed + 1)
    clean = H.forward(torch.tensor(f_true, dtype=torch.float32)) * 20
    g = torch.poisson(clean, generator=gen)
    rec["projections"] = g.numpy()
    s = None
    if additive:
        s = torch.full(g.shape, float(clean.mean()) * 0.1)
        rec["additive"] = s.numpy()
    iterates = []

    class Keep:
        def run(self, obj, n_iter, n_subset):
            iterates.append(obj.clone().numpy())
            return obj

        def finalize(self, obj):
            pass

    lik = PoissonLogLikelihood(H, g, additive_term=s)
    if bsrem:
        prior = RelativeDifferencePrior(beta=0.3, gamma=2)
        alg = BSREM(lik, prior=prior)
        rec["beta"], rec["gamma"] = 0.3, 2.0
    else:
        alg = OSEM(lik)
    alg(n_iters, n_subsets, callback=Keep())
    rec["iterates"] = np.stack(iterates)
    rec["norm_bps"] = np.stack([nb.numpy() for nb in lik.norm_BPs])
    np.savez_compressed(os.path.join(out, f"{name}.npz"), **rec)
    print("wrote", name)


def rdp_case(out):
    set_precision(torch.float32)
    rng = np.random.default_rng(7)
    shape = (10, 12, 9)
    dr = (0.4, 0.4, 0.5)
    f = rng.random(shape) * 5 + 0.01
    f[2:4, 3:7, 1:5] = 0.0
    prior = RelativeDifferencePrior(beta=0.3, gamma=2)
    om = SPECTObjectMeta(list(dr), shape)
    prior.set_object_meta(om)
    prior.set_object(torch.tensor(f, dtype=torch.float32))
    prior.set_beta_scale(0.25)
    grad = prior(derivative_order=1).numpy()
    value = prior(derivative_order=0)
    np.savez_compressed(os.path.join(out, "rdp.npz"), object=f, dr=np.array(dr), beta=0.3,
                        gamma=2.0, beta_scale=0.25, grad=grad, value=value)
    print("wrote rdp")


def pet_meta_case(out):
    set_precision(torch.float32)
    rec = {}
    for nb, rng_mm, fwhm in ((13, 650.0, 58.5), (12, 600.0, 40.0)):
        m = PETTOFMeta(nb, rng_mm, fwhm)
        rec[f"tof_{nb}"] = np.array([float(m.bin_width), float(m.sigma), float(m.center_offset),
                                     float(m.n_sigmas)])
    info = dict(crystalTransNr=1, crystalTransSpacing=4.0, submoduleTransNr=1,
                submoduleTransSpacing=0.0, moduleTransNr=1, moduleTransSpacing=0.0,
                rsectorTransNr=60, crystalAxialNr=8, crystalAxialSpacing=4.0,
                submoduleAxialNr=1, submoduleAxialSpacing=0.0, moduleAxialNr=1,
                moduleAxialSpacing=0.0, rsectorAxialNr=1, radius=120.0,
                firstCrystalAxis=1, NrCrystalsPerRing=60, NrRings=8)
    rec["lut_small"] = pet_shared.get_scanner_LUT(info).numpy()
    rec["lut_small_info"] = np.array([60, 8, 120.0, 4.0])
    np.savez_compressed(os.path.join(out, "pet_meta.npz"), **rec)
    print("wrote pet_meta")


def pet_sino_case(out):
    """Sinogram geometry tables and listmode -> sinogram binning of a small scanner
    (io/PET/shared.py:7-272)."""
    set_precision(torch.float32)
    info = dict(crystalTransNr=1, crystalTransSpacing=4.0, submoduleTransNr=1,
                submoduleTransSpacing=0.0, moduleTransNr=1, moduleTransSpacing=0.0,
                rsectorTransNr=60, crystalAxialNr=8, crystalAxialSpacing=4.0,
                submoduleAxialNr=1, submoduleAxialSpacing=0.0, moduleAxialNr=1,
                moduleAxialSpacing=0.0, rsectorAxialNr=1, radius=120.0,
                firstCrystalAxis=1, NrCrystalsPerRing=60, NrRings=8, min_rsector_difference=0)
    rec = {}
    lor, sidx = pet_shared.sinogram_coordinates(info)
    rec["lor_coordinates"] = lor.numpy()
    rec["sinogram_index"] = sidx.numpy()
    det, ring = pet_shared.sinogram_to_spatial(info)
    rec["detector_coordinates"] = det.numpy()
    rec["ring_coordinates"] = ring.numpy()
    g = torch.Generator().manual_seed(31)
    n_det = 60 * 8
    ids = torch.randint(0, n_det, (4000, 2), generator=g)
    ids = ids[ids[:, 0] != ids[:, 1]]
    tof = torch.randint(0, 13, (ids.shape[0], 1), generator=g)
    w = torch.rand(ids.shape[0], generator=g)
    rec["events"] = torch.cat([ids, tof], 1).numpy()
    rec["weights"] = w.numpy()
    rec["sino"] = pet_shared.listmode_to_sinogram(ids, info).numpy()
    rec["sino_w"] = pet_shared.listmode_to_sinogram(ids, info, weights=w).numpy()
    rec["sino_norm"] = pet_shared.listmode_to_sinogram(ids, info, weights=w,
                                                       normalization=True).numpy()
    tm = PETTOFMeta(13, 650.0, 58.5)
    rec["sino_tof"] = pet_shared.listmode_to_sinogram(torch.cat([ids, tof], 1), info,
                                                      tof_meta=tm).numpy()
    np.savez_compressed(os.path.join(out, "pet_sino.npz"), **rec)
    print("wrote pet_sino", {k: v.shape for k, v in rec.items()})


def kem_filter_case(out):
    """GaussianFilter (transforms/shared/filters.py), KEMTransform (transforms/shared/kem.py)
    and KEMSystemMatrix over a SPECT system matrix (projectors/shared/kem_system_matrix.py)."""
    from pytomography.metadata import ObjectMeta
    from pytomography.transforms.shared import GaussianFilter, KEMTransform
    from pytomography.projectors.shared import KEMSystemMatrix
    set_precision(torch.float32)
    g = torch.Generator().manual_seed(41)
    shape, dr = (14, 12, 10), (0.4, 0.5, 0.45)
    om = ObjectMeta(list(dr), shape)
    f = torch.rand(shape, generator=g) + 0.2
    rec = {"object": f.numpy(), "shape": np.array(shape), "dr": np.array(dr)}
    for fwhm, ns in ((1.2, 3.0), (0.7, 2.0)):
        gf = GaussianFilter(fwhm, n_sigmas=ns)
        gf.configure(om, None)
        rec[f"gauss_{fwhm}_{ns}"] = gf(f.to(pt.device)).cpu().numpy()
    s1 = torch.rand(shape, generator=g)
    s2 = (torch.rand(shape, generator=g) > 0.5).to(torch.float32) * 3.0
    rec["support1"], rec["support2"] = s1.numpy(), s2.numpy()
    kem = KEMTransform([s1, s2], support_kernels_params=[[0.3], [1.0]],
                       distance_kernel_params=[0.6], size=5)
    kem.configure(om, None)
    rec["kem_fwd"] = kem.forward(f.to(pt.device)).cpu().numpy()
    kem3 = KEMTransform([s1], support_kernels_params=[[0.2]], distance_kernel_params=[0.5],
                        size=3, top_N=10)
    kem3.configure(om, None)
    rec["kem3_top10_fwd"] = kem3.forward(f.to(pt.device)).cpu().numpy()
    # KEM over a small SPECT system matrix with attenuation
    sshape, sdr = (12, 12, 8), (0.48, 0.48, 0.48)
    angles = [float(a) for a in np.linspace(0, 360, 9)[:-1]]
    om2 = SPECTObjectMeta(list(sdr), sshape)
    pm2 = SPECTProjMeta(sshape[1:], list(sdr[:2]), angles, radii=[20.0] * len(angles))
    mu = torch.rand(sshape, generator=g) * 0.1
    H = SPECTSystemMatrix([SPECTAttenuationTransform(mu.to(pt.device))], [], om2, pm2)
    sup = torch.rand(sshape, generator=g)
    kem2 = KEMTransform([sup], support_kernels_params=[[0.5]], distance_kernel_params=[1.0],
                        size=3)
    K = KEMSystemMatrix(H, kem2)
    alpha = torch.rand(sshape, generator=g) + 0.1
    proj = torch.rand((len(angles), *sshape[1:]), generator=g)
    rec.update(spect_mu=mu.numpy(), spect_support=sup.numpy(), spect_angles=np.array(angles),
               spect_alpha=alpha.numpy(), spect_proj=proj.numpy(),
               kem_spect_fwd=K.forward(alpha.to(pt.device)).cpu().numpy(),
               kem_spect_bwd=K.backward(proj.to(pt.device)).cpu().numpy())
    K.set_n_subsets(2)
    rec["kem_spect_norm1"] = K.compute_normalization_factor(1).cpu().numpy()
    np.savez_compressed(os.path.join(out, "kem_filter.npz"), **rec)
    print("wrote kem_filter", sorted(rec))


def uncertainty_case(out):
    """compute_uncertainty over a DataStorageCallback (preconditioned_gradient_ascent.py:
    170-299, callbacks/data_saving.py) for OSEM, OSEM with a post-reconstruction Gaussian
    filter, and BSREM with the RDP prior (its second derivative)."""
    from pytomography.callbacks import DataStorageCallback
    from pytomography.transforms.shared import GaussianFilter
    shape, dr = (16, 16, 10), (0.48, 0.48, 0.48)
    angles = [float(a) for a in np.linspace(0, 360, 13)[:-1]]
    radius, seed = 20.0, 51
    f_true, mu_np = ellipsoid_phantom(shape, dr, seed, n_ell=2)
    set_precision(torch.float32)
    om = SPECTObjectMeta(list(dr), tuple(shape))
    pm = SPECTProjMeta((shape[1], shape[2]), list(dr[:2]), angles, radii=[radius] * len(angles))
    H = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(mu_np, dtype=torch.float32)),
                           SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm)
    g = torch.poisson(H.forward(torch.tensor(f_true, dtype=torch.float32)) * 20,
                      generator=torch.Generator().manual_seed(seed + 1))
    mask = torch.zeros(shape, dtype=torch.bool)
    mask[5:11, 4:10, 3:7] = True
    rec = {"shape": np.array(shape), "dr": np.array(dr), "angles": np.array(angles),
           "radius": radius, "mu": mu_np, "projections": g.numpy(), "mask": mask.numpy()}
    for name, bsrem in (("osem", False), ("bsrem", True)):
        lik = PoissonLogLikelihood(H, g)
        if bsrem:
            alg = BSREM(lik, prior=RelativeDifferencePrior(beta=0.3, gamma=2))
        else:
            alg = OSEM(lik)
        cb = DataStorageCallback(lik, torch.clone(alg.object_prediction))
        recon = alg(2, 3, callback=cb)
        rec[f"{name}_recon"] = recon.numpy()
        a_abs, a_pct = alg.compute_uncertainty(mask, cb, return_pct=True)
        rec[f"{name}_unc"] = np.array([a_abs, a_pct])
        rec[f"{name}_unc_sub3"] = np.array(alg.compute_uncertainty(mask, cb, subiteration_number=3))
        if not bsrem:
            gf = GaussianFilter(0.8)
            gf.configure(om, pm)
            # the filter convolves the mask, so it has to be a float mask
            rec["osem_unc_filtered"] = np.array(alg.compute_uncertainty(
                mask.to(torch.float32), cb, post_recon_filter=gf))
    np.savez_compressed(os.path.join(out, "uncertainty.npz"), **rec)
    print("wrote uncertainty", {k: v for k, v in rec.items() if k.endswith(("unc", "sub3", "filtered"))})


def multibed_case(out):
    """PGAAMultiBedSPECT (preconditioned_gradient_ascent.py:550-600) over three bed positions
    with stitch_multibed (io/SPECT/dicom.py:599-653).  The bed z positions and slice spacing
    that the reference reads from DICOM headers are given by stand-in header objects."""
    from pytomography.algorithms import PGAAMultiBedSPECT
    from pytomography.io.SPECT import dicom as ref_dicom
    shape, dr = (16, 16, 10), (0.48, 0.48, 0.48)
    angles = [float(a) for a in np.linspace(0, 360, 13)[:-1]]
    z_mm = [57.6, 0.0, 28.8]  # unsorted on purpose: the stitching sorts by z
    spacing_mm = 4.8

    class _Pos:
        def __init__(self, z):
            self.ImagePositionPatient = [0.0, 0.0, z]

    class _Header:
        def __init__(self, z):
            self.DetectorInformationSequence = [_Pos(z)]
            self.PixelSpacing = [spacing_mm, spacing_mm]
            self.Rows = shape[0]

    headers = {f"bed{i}": _Header(z) for i, z in enumerate(z_mm)}
    ref_dicom.pydicom.dcmread = lambda f: headers[f]
    set_precision(torch.float32)
    rec = {"shape": np.array(shape), "dr": np.array(dr), "angles": np.array(angles),
           "z_mm": np.array(z_mm), "spacing_mm": spacing_mm}
    algs = []
    for b in range(3):
        f_true, mu_np = ellipsoid_phantom(shape, dr, 60 + b, n_ell=2)
        om = SPECTObjectMeta(list(dr), shape)
        pm = SPECTProjMeta(shape[1:], list(dr[:2]), angles, radii=[20.0] * len(angles))
        H = SPECTSystemMatrix([SPECTAttenuationTransform(torch.tensor(mu_np, dtype=torch.float32)),
                               SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))], [], om, pm)
        g = torch.poisson(H.forward(torch.tensor(f_true, dtype=torch.float32)) * 20,
                          generator=torch.Generator().manual_seed(70 + b))
        rec[f"mu{b}"], rec[f"proj{b}"] = mu_np, g.numpy()
        algs.append(OSEM(PoissonLogLikelihood(H, g)))
    mb = PGAAMultiBedSPECT([f"bed{i}" for i in range(3)], algs)
    rec["stitched"] = mb(2, 3).numpy()
    rec["beds"] = np.stack([a.object_prediction.numpy() for a in algs])
    np.savez_compressed(os.path.join(out, "multibed.npz"), **rec)
    print("wrote multibed", rec["stitched"].shape)


def starguide_case(out):
    """StarGuideSystemMatrix (projectors/SPECT/starguide_system_matrix.py:12-230) with
    StarGuideProjMeta (metadata/SPECT/starguide_metadata.py): 12 detectors at 3 angles with
    per-detector offsets, radii and times; attenuation and PSF on the unpadded frame
    (assume_padded=False, which this path needs)."""
    from pytomography.metadata.SPECT import StarGuideProjMeta
    from pytomography.projectors.SPECT import StarGuideSystemMatrix
    set_precision(torch.float32)
    shape, dr = (32, 32, 8), (0.5, 0.5, 0.5)
    rng = np.random.default_rng(81)
    angles = np.array([10.0, 100.0, 215.0] * 4)
    offsets = rng.uniform(-3.0, 3.0, 12)
    radii = rng.uniform(15.0, 25.0, 12)
    times = rng.uniform(500.0, 1500.0, 12)
    f_true, mu_np = ellipsoid_phantom(shape, dr, 82, n_ell=2)
    om = SPECTObjectMeta(list(dr), shape)
    rec = {"shape": np.array(shape), "dr": np.array(dr), "angles": angles, "offsets": offsets,
           "radii": radii, "times": times, "object": f_true, "mu": mu_np}
    g = torch.Generator().manual_seed(83)
    proj = torch.rand((12, 16, shape[2]), generator=g)
    rec["proj"] = proj.numpy()
    for name, with_psf in (("att", False), ("att_psf", True)):
        pm = StarGuideProjMeta((12, 16, shape[2]), torch.tensor(angles, dtype=torch.float32),
                               times=torch.tensor(times, dtype=torch.float32),
                               offsets=torch.tensor(offsets, dtype=torch.float32),
                               radii=[float(r) for r in radii])
        ts = [SPECTAttenuationTransform(torch.tensor(mu_np, dtype=torch.float32),
                                        assume_padded=False)]
        if with_psf:
            ts.append(SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)), assume_padded=False))
        H = StarGuideSystemMatrix(om, pm, obj2obj_transforms=ts)
        f = torch.tensor(f_true, dtype=torch.float32)
        rec[f"{name}_fwd"] = H.forward(f).numpy()
        rec[f"{name}_bwd"] = H.backward(proj).numpy()
        H.set_n_subsets(2)
        rec[f"{name}_subsets"] = np.concatenate([x.numpy() for x in H.subset_indices_array])
        rec[f"{name}_fwd_s1"] = H.forward(f, 1).numpy()
        rec[f"{name}_bwd_s1"] = H.backward(H.get_projection_subset(proj, 1), 1).numpy()
        rec[f"{name}_norm_s0"] = H.compute_normalization_factor(0).numpy()
    np.savez_compressed(os.path.join(out, "starguide.npz"), **rec)
    print("wrote starguide", rec["att_psf_fwd"].shape, rec["att_subsets"])


def theta_case(out):
    """Sampling matrices of the restated kornia rotation, for pinning the host tables."""
    rec = {}
    angles = torch.tensor([0.0, 3.7, 45.0, 90.0, 97.0, 180.0, 222.5, 270.0, 333.3, -270.0, -93.0],
                          dtype=torch.float32)
    for size in (23, 24, 92, 182):
        th = refharness.kornia_sampling_matrix(
            angles, torch.tensor([(size - 1) / 2.0, (size - 1) / 2.0]).expand(len(angles), 2),
            size, size)
        rec[f"theta_{size}"] = th.reshape(len(angles), 6).numpy()
        rec[f"lin_{size}"] = torch.linspace(-1, 1, size).numpy()
    rec["angles"] = angles.numpy()
    np.savez_compressed(os.path.join(out, "theta.npz"), **rec)
    print("wrote theta")


def autograd_case(out):
    """Gradient of the Poisson NLL through the reference forward projector, by torch
    autograd through its undecorated transforms (the reference wraps them in no_grad)."""
    from pytomography.transforms.shared import RotationTransform
    set_precision(torch.float64)
    shape, dr = (16, 16, 10), (0.48, 0.48, 0.48)
    angles = [float(a) for a in np.linspace(0, 360, 9)[:-1]]
    f_np, mu_np = ellipsoid_phantom(shape, dr, 31)
    f_np = f_np + 0.2
    om = SPECTObjectMeta(list(dr), shape)
    pm = SPECTProjMeta(shape[1:], list(dr[:2]), angles, radii=[20.0] * len(angles))
    att = SPECTAttenuationTransform(torch.tensor(mu_np))
    psf = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)))
    H = SPECTSystemMatrix([att, psf], [], om, pm)
    rng = np.random.default_rng(32)
    g_np = rng.poisson(H.forward(torch.tensor(f_np)).numpy() * 3).astype(np.float64)
    saved = {}
    for cls, name in ((RotationTransform, "backward"), (type(att), "forward"),
                      (type(psf), "forward")):
        saved[(cls, name)] = getattr(cls, name)
        setattr(cls, name, getattr(cls, name).__wrapped__)
    try:
        f = torch.tensor(f_np, requires_grad=True)
        pred = H.forward(f)
        g = torch.tensor(g_np)
        nll = (pred - g * torch.log(pred + 1e-11)).sum()
        nll.backward()
        grad = f.grad.numpy()
    finally:
        for (cls, name), fn in saved.items():
            setattr(cls, name, fn)
    set_precision(torch.float32)
    np.savez_compressed(os.path.join(out, "autograd.npz"), shape=np.array(shape),
                        dr=np.array(dr), angles=np.array(angles), radii=np.full(len(angles), 20.0),
                        object=f_np, mu=mu_np, projections=g_np, nll=float(nll), grad=grad)
    print("wrote autograd")


def plugins_case(out):
    """The two obj2obj plugins called on their own, one projection index at a time, on
    seeded objects already in the detector frame (SPECTAttenuationTransform.forward /
    backward, attenuation.py:72-115; SPECTPSFTransform.forward / backward, psf.py:199-231),
    in the padded frame of SPECTSystemMatrix and in the unpadded frame
    (assume_padded=False) of the StarGuide system matrix."""
    shape, dr = (14, 14, 8), (0.45, 0.45, 0.5)
    angles = [0.0, 33.0, 90.0, 145.5, 200.0, 271.0, 318.0]
    radii = [21.0, 25.0, 21.0, 23.0, 25.0, 21.0, 24.5]
    f_np, mu_np = ellipsoid_phantom(shape, dr, seed=31)
    rng = np.random.default_rng(32)
    pad = compute_pad_size(shape[0])
    L = shape[0] + 2 * pad
    rec = {"shape": np.array(shape), "dr": np.array(dr), "angles": np.array(angles),
           "radii": np.array(radii), "mu": mu_np, "pad": pad}
    x_pad = (rng.random((L, L, shape[2])) * 4).astype(np.float32)
    x_unp = (rng.random(shape) * 4).astype(np.float32)
    rec["x_padded"], rec["x_unpadded"] = x_pad, x_unp
    idx = [0, 3, 5]
    rec["indices"] = np.array(idx)
    for prec, dt in (("f32", torch.float32), ("f64", torch.float64)):
        set_precision(dt)
        om = SPECTObjectMeta(list(dr), tuple(shape))
        pm = SPECTProjMeta((shape[1], shape[2]), list(dr[:2]), list(angles), radii=list(radii))
        for frame, x_np, padded in (("pad", x_pad, True), ("unpad", x_unp, False)):
            att = SPECTAttenuationTransform(torch.tensor(mu_np, dtype=dt), assume_padded=padded)
            psf2 = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11)), assume_padded=padded)
            psf1 = SPECTPSFTransform(SPECTPSFMeta((0.03, 0.11), kernel_dimensions="1D"),
                                     assume_padded=padded)
            for t in (att, psf2, psf1):
                t.configure(om, pm)
            x = torch.tensor(x_np, dtype=dt)
            for i in idx:
                ai = torch.tensor(i)
                outs = {"att_fwd": att.forward(x, ai), "att_bwd": att.backward(x, ai),
                        "psf_fwd": psf2.forward(x, ai), "psf_bwd": psf2.backward(x, ai),
                        "psf1d_fwd": psf1.forward(x, ai)}
                for k, v in outs.items():
                    if prec == "f64" and (frame != "pad" or k.endswith("bwd")):
                        continue
                    rec[f"{k.replace('_', '_' + frame + '_', 1)}_{i}_{prec}"] = v.detach().numpy()
    set_precision(torch.float32)
    np.savez_compressed(os.path.join(out, "plugins.npz"), **rec)
    print("wrote plugins", L)


def pet_fov_case(out):
    """PETLMSystemMatrix._get_object_initial and _get_prior_FOV_scale
    (petlm_system_matrix.py:59-89) for the small scanner of pet_meta and a 40 x 36 x 16
    image at 2 mm: the axial field of view zeroes / tapers the outer z slices.  The
    methods only read the object and scanner geometry, so they run on a stand-in instance
    (the constructor would compute a sensitivity image through parallelproj)."""
    from types import SimpleNamespace
    from pytomography.metadata import ObjectMeta
    from pytomography.projectors.PET import PETLMSystemMatrix
    set_precision(torch.float32)
    info = dict(crystalTransNr=1, crystalTransSpacing=4.0, submoduleTransNr=1,
                submoduleTransSpacing=0.0, moduleTransNr=1, moduleTransSpacing=0.0,
                rsectorTransNr=60, crystalAxialNr=8, crystalAxialSpacing=4.0,
                submoduleAxialNr=1, submoduleAxialSpacing=0.0, moduleAxialNr=1,
                moduleAxialSpacing=0.0, rsectorAxialNr=1, radius=120.0,
                firstCrystalAxis=1, NrCrystalsPerRing=60, NrRings=8)
    lut = pet_shared.get_scanner_LUT(info)
    shape, dr = (40, 36, 16), (2.0, 2.0, 2.0)
    me = SimpleNamespace(object_meta=ObjectMeta(list(dr), shape),
                         proj_meta=SimpleNamespace(scanner_lut=lut), FOV_scale_enabled=True)
    init = PETLMSystemMatrix._get_object_initial(me, device="cpu").numpy()
    fov = PETLMSystemMatrix._get_prior_FOV_scale(me).cpu().numpy()
    np.savez_compressed(os.path.join(out, "pet_fov.npz"), shape=np.array(shape),
                        dr=np.array(dr), object_initial=init, fov_scale=fov)
    print("wrote pet_fov", float(init.mean()), float(fov.mean()))


def camera_path_case(out):
    """SPECTSystemMatrix._get_object_initial with object_initial_based_on_camera_path
    (spect_system_matrix.py:38-56): ones, zeroed in every angle's rotated frame behind the
    camera orbit (radii smaller than half the object width)."""
    shape, dr = (16, 16, 8), (0.5, 0.5, 0.5)
    angles = [0.0, 40.0, 95.0, 150.0, 200.0, 245.0, 300.0, 330.0]
    radii = [3.6, 2.6, 3.1, 2.4, 3.9, 2.9, 4.6, 2.2]
    om = SPECTObjectMeta(list(dr), shape)
    pm = SPECTProjMeta((shape[1], shape[2]), list(dr[:2]), list(angles), radii=list(radii))
    H = SPECTSystemMatrix([], [], om, pm, object_initial_based_on_camera_path=True)
    init = H._get_object_initial(device="cpu").numpy()
    np.savez_compressed(os.path.join(out, "camera_path.npz"), shape=np.array(shape),
                        dr=np.array(dr), angles=np.array(angles), radii=np.array(radii),
                        object_initial=init)
    print("wrote camera_path", float(init.mean()))


CASES = {}


def main():
    out = HERE
    only = set(sys.argv[1:])
    if only:
        for name in sorted(only):
            {"plugins": plugins_case, "camera_path": camera_path_case,
             "pet_fov": pet_fov_case}[name](out)
        return
    plugins_case(out)
    camera_path_case(out)
    pet_fov_case(out)
    autograd_case(out)
    theta_case(out)
    torch.manual_seed(0)
    spect_case("spect_even", (16, 16, 12), (0.48, 0.48, 0.48),
               [float(a) for a in np.linspace(0, 360, 11)[:-1]],
               [25.0 if i % 2 == 0 else 21.0 for i in range(10)],
               ["none", "att", "psf", "att+psf", "psf+att", "att+psf1d"], seed=11, out=out)
    spect_case("spect_odd", (15, 15, 10), (0.442, 0.442, 0.5),
               [3.7, 51.2, 97.0, 180.0, 222.5, 270.0, 333.3],
               [22.0, 22.0, 19.0, 22.0, 23.5, 22.0, 19.0],
               ["none", "att+psf"], seed=12, out=out)
    osem_case("osem_small", (16, 16, 10), (0.48, 0.48, 0.48),
              [float(a) for a in np.linspace(0, 360, 13)[:-1]], 20.0, 2, 3, seed=21, out=out)
    osem_case("osem_additive", (14, 14, 8), (0.5, 0.5, 0.5),
              [float(a) for a in np.linspace(0, 360, 9)[:-1]], 18.0, 2, 2, seed=22, out=out,
              additive=True)
    osem_case("bsrem_small", (16, 16, 10), (0.48, 0.48, 0.48),
              [float(a) for a in np.linspace(0, 360, 13)[:-1]], 20.0, 2, 3, seed=23, out=out,
              bsrem=True)
    rdp_case(out)
    pet_meta_case(out)
    pet_sino_case(out)
    kem_filter_case(out)
    uncertainty_case(out)
    multibed_case(out)
    starguide_case(out)
    print("pad sizes", {n: compute_pad_size(n) for n in (15, 16, 64, 96, 128)})


if __name__ == "__main__":
    main()
