"""Parity report at the benchmark workloads' full sizes (run on a GPU machine):

    python tests/parity_report.py [--out report.md]

For every workload the float32 CUDA path is compared with

* the float64 C oracle (``oracle/``), which restates the reference's algorithm; and
* the reference's per-call sequence restated in plain PyTorch float32 on the GPU
  (``tests/torch_reference.py``, itself pinned to the golden fixtures made from the
  reference), for the SPECT workloads.

Figures are relative L2 errors: per projection (the maximum over the projections
compared), per back projection, per OSEM iterate (the maximum over the iterates
compared), per object gradient, and per PET listmode forward / back projection.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from torch_reference import TorchReferenceProjector  # noqa: E402


def rel(a, b) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def per_row(a, b) -> float:
    return max(rel(a[i], b[i]) for i in range(a.shape[0]))


def spect_oracle(w, precision="f64"):
    order = "a" + ("p" if w.psf is not None else "")
    return oracle.SpectOracle(w.shape, w.dr, w.angles, [w.radius] * len(w.angles), mu=w.mu,
                              psf=w.psf, order=order, precision=precision)


def spect_rows(name, w, n_sub, fwd_subsets, osem_subiters_oracle, osem_iters_torch, rows):
    from pytomography_gb300 import synthetic
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    H = synthetic.build_system_matrix(w)
    g = synthetic.poisson_projections(H, w)
    H.set_n_subsets(n_sub)
    R = TorchReferenceProjector(H)
    o = spect_oracle(w)
    f = torch.tensor(w.activity, dtype=torch.float32, device="cuda")
    e_fo = e_ft = e_bo = e_bt = e_ao = 0.0
    rng = np.random.default_rng(11)
    for k in fwd_subsets:
        idx = H.subset_indices_array[k].cpu().numpy()
        ours = H.forward(f, k).cpu().numpy()
        e_fo = max(e_fo, per_row(ours, o.forward(w.activity, idx)))
        e_ft = max(e_ft, per_row(ours, R.forward(f, k).cpu().numpy()))
        gg = rng.random(ours.shape) + 0.5
        gt = torch.tensor(gg, dtype=torch.float32, device="cuda")
        ob = H.backward(gt, k).cpu().numpy()
        e_bo = max(e_bo, rel(ob, o.backward(gg, idx)))
        e_bt = max(e_bt, rel(ob, R.backward(gt, k).cpu().numpy()))
        e_ao = max(e_ao, rel(H.backward_adjoint(gt, k).cpu().numpy(), o.adjoint(gg, idx)))
    rows.append((name, "forward projection (per projection, max)", e_fo, e_ft))
    rows.append((name, "back projection, reference operator", e_bo, e_bt))
    rows.append((name, "back projection, exact adjoint", e_ao, None))
    # OSEM iterates: fused CUDA path vs the oracle (first sub-iterations) and vs the
    # PyTorch sequence (whole iterations)
    gd = g.to("cuda")
    lik = PoissonLogLikelihood(H, gd)
    lik._set_n_subsets(n_sub)
    fo = torch.ones(w.shape, device="cuda")
    ft = torch.ones(w.shape, device="cuda")
    e_ot = 0.0
    ours_its = []
    for it in range(osem_iters_torch):
        for k in range(n_sub):
            H.osem_step(fo, gd, None, lik._get_normBP(k), k)
            ft = R.osem_subiteration(ft, gd, None, lik._get_normBP(k), k)
            e_ot = max(e_ot, rel(fo.cpu().numpy(), ft.cpu().numpy()))
            if len(ours_its) < osem_subiters_oracle:
                ours_its.append(fo.cpu().numpy())
    e_oo = None
    if osem_subiters_oracle:
        subs = oracle.subsets(len(w.angles), n_sub)
        fr = np.ones(w.shape)
        e_oo = 0.0
        gn = g.numpy().astype(np.float64)
        for m in range(osem_subiters_oracle):
            k = subs[m % n_sub]
            norm = o.backward(np.ones((len(k),) + gn.shape[1:]), k)
            pred = o.forward(fr, k)
            grad = o.backward(gn[k] / (pred + oracle.DELTA), k) - norm
            fr = fr + fr * (1 / (norm + oracle.DELTA)) * grad
            fr[fr <= 0] = 0
            e_oo = max(e_oo, rel(ours_its[m], fr))
    rows.append((name, f"OSEM iterates ({osem_subiters_oracle} sub-its vs oracle, "
                       f"{osem_iters_torch * n_sub} vs PyTorch)", e_oo, e_ot))
    return H


def gradient_rows(rows):
    """Poisson-NLL gradient through the autograd Function vs torch autograd through the
    PyTorch restatement (one 12-angle subset) and vs the float64 oracle adjoint."""
    from pytomography_gb300 import synthetic
    from pytomography_gb300.autograd import poisson_nll
    w = synthetic.config2(seed=10)
    H = synthetic.build_system_matrix(w)
    g = synthetic.poisson_projections(H, w).to("cuda")
    H.set_n_subsets(10)
    R = TorchReferenceProjector(H)
    f0 = torch.tensor(w.activity, dtype=torch.float32, device="cuda") * 0.7 + 0.3
    k = 4
    idx = H.subset_indices_array[k]
    gk = g[idx]
    f1 = f0.clone().requires_grad_(True)
    poisson_nll(f1, H, gk, subset_idx=k).backward()
    f2 = f0.clone().requires_grad_(True)
    pred = R.forward(f2, k)
    (pred - gk * torch.log(pred + 1e-11)).sum().backward()
    o = spect_oracle(w)
    fn = f0.double().cpu().numpy()
    i = idx.cpu().numpy()
    p = o.forward(fn, i)
    grad64 = o.adjoint(1.0 - gk.double().cpu().numpy() / (p + oracle.DELTA), i)
    ours = f1.grad.cpu().numpy()
    rows.append(("8 x 128^3 gradients", "Poisson-NLL object gradient (one subset)",
                 rel(ours, grad64), rel(ours, f2.grad.cpu().numpy())))


def pet_rows(rows, n_events=200_000):
    from pytomography_gb300 import synthetic
    from pytomography_gb300.metadata.PET import PETTOFMeta
    w = synthetic.config3(n_events=n_events)
    H = synthetic.build_pet_system_matrix(w)
    tm = PETTOFMeta(*w.tof)
    o = oracle.PetLMOracle(w.shape, w.voxel_mm, H.proj_meta.scanner_lut.numpy(),
                           tof=(w.tof[0], float(tm.bin_width), float(tm.sigma),
                                float(tm.center_offset), float(tm.n_sigmas)))
    rng = np.random.default_rng(12)
    img = rng.random(w.shape) + 0.1
    fwd = H.forward(torch.tensor(img, dtype=torch.float32, device="cuda")).cpu().numpy()
    ref = o.forward(img, w.events)
    proj = rng.random(w.events.shape[0]) + 0.1
    bwd = H.backward(torch.tensor(proj, dtype=torch.float32, device="cuda")).cpu().numpy()
    rows.append(("PET TOF listmode", f"forward projection ({n_events} events)", rel(fwd, ref),
                 None))
    rows.append(("PET TOF listmode", "back projection", rel(bwd, o.backward(proj, w.events)),
                 None))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    from pytomography_gb300 import synthetic
    t0 = time.time()
    rows = []
    spect_rows("64^3 x 64, att", synthetic.config1(), 8, [0, 5], 4, 4, rows)
    spect_rows("128^3 x 120, att+PSF", synthetic.config2(), 10, [0, 7], 2, 1, rows)
    gradient_rows(rows)
    ws = synthetic.config5()
    seen = set()
    for w in ws:
        key = w.shape[0]
        if key in seen:
            continue
        seen.add(key)
        spect_rows(f"serving {w.shape[0]}^3 x {len(w.angles)}", w, 10, [3], 1, 1, rows)
    pet_rows(rows)
    fmt = lambda v: "-" if v is None else f"{v:.2e}"  # noqa: E731
    lines = ["| workload | quantity | vs float64 oracle | vs PyTorch reference sequence |",
             "|---|---|---|---|"]
    for name, what, a, b in rows:
        lines.append(f"| {name} | {what} | {fmt(a)} | {fmt(b)} |")
    lines.append("")
    lines.append(f"({time.time() - t0:.0f} s; GPU {torch.cuda.get_device_name()})")
    text = "\n".join(lines)
    print(text)
    if args.out:
        with open(args.out, "w") as fh:
            fh.write(text + "\n")


if __name__ == "__main__":
    main()
