"""Benchmark: OSEM sub-iterations/s at 128^3 x 120 angles (attenuation + PSF) on one GB300.

Workload (the 128^3 / 120-angle configuration): float32 object 128x128x128 at 4.42 mm,
seeded ellipsoid phantom with three 8:1 hot spheres, mu 0-0.2 cm^-1 (lungs 0.04), 120
angles over 360 deg at 22 cm, PSF sigma(d) = 0.03 d + 0.11 cm, Poisson projections,
10 subsets of 12 angles.  A "step" is one OSEM sub-iteration.

  value    : fused sub-iterations (forward with ratio epilogue, back-projection with
             fused update) replayed from captured CUDA graphs, inputs resident in HBM
  plain    : the per-call drop-in path (forward, torch ratio, backward, torch update)
  torch_reference : the reference's per-call GPU sequence restated in plain PyTorch
             float32 (per angle: pad, grid_sample rotation of object and mu, cumsum
             attenuation, grouped conv1d PSF, sum; tests/torch_reference.py)
  e2e      : OSEM(likelihood)(4, 10) through the public API from host tensors
             (system matrix construction, H2D of projections and mu, normalisation,
             40 sub-iterations, D2H of the result), reported per sub-iteration
  roofline : forward projector (k_fwd_psf + k_reduce), algorithmic bytes per launch from
             the padded-volume model 12 x (4P(1+a) + 4Q), P = 182*182*128, Q = 182*128
  cpu_baseline : the float32 C oracle port of the same sub-iteration on the host cores

``--impl reference`` times the CPU implementation of the path (the oracle port, all host
threads) on the same workload and prints the same JSON line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "OSEM subiter/s at 128^3x120 ang (att+PSF)"
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one 12-angle k_fwd_psf launch
# of this workload, from a separate ncu capture of the same kernel (a constant: this
# script does not run ncu)
FWD_DRAM_BYTES_PER_LAUNCH = 114.981e6 + 3.262e6
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Whole-job time: the maximum of a per-rank value over all ranks (replicas)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(PEAKS) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def alg_bytes_subiter(n=128, n_sel=12, att=1):
    pad = int(np.ceil((np.sqrt(2) * n - n) / 2))
    Lp = n + 2 * pad
    P, Q, V = Lp * Lp * n, Lp * n, n * n * n
    fwd = n_sel * (4 * P * (1 + att) + 4 * Q)
    bwd = n_sel * (4 * Q + 4 * att * P + 8 * P)
    return fwd, bwd, fwd + bwd + 16 * n_sel * n * n + 16 * V


class Clocks:
    """SM clock and clock-event reasons of this process's GPU, sampled about every
    millisecond while the timed region runs (NVML through ctypes, read-only queries;
    nvidia-smi at 100 ms as a fallback).  The device is addressed by its UUID, so the
    sampler reads the leased GPU even when CUDA_VISIBLE_DEVICES renumbers it."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, path, device):
        import torch
        self.path = path
        self.samples = []  # (sm MHz, reason bits)
        self.max_mhz = None
        self.source = None
        try:
            self.uuid = "GPU-" + str(torch.cuda.get_device_properties(device).uuid)
        except Exception:
            self.uuid = None
        self._nvml = None
        self._thread = None
        self._proc = None

    def _nvml_open(self):
        import ctypes
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0 or not self.uuid:
            return None
        h = ctypes.c_void_p()
        if nv.nvmlDeviceGetHandleByUUID(self.uuid.encode(), ctypes.byref(h)) != 0:
            return None
        mx = ctypes.c_uint(0)
        if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:  # 1 = SM clock
            self.max_mhz = float(mx.value)
        fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        return nv, h, fn

    def __enter__(self):
        import ctypes
        import threading
        try:
            self._nvml = self._nvml_open()
        except Exception:
            self._nvml = None
        if self._nvml is not None:
            nv, h, reasons_fn = self._nvml
            self.source = "nvml, ~1 ms"
            self._stop = threading.Event()

            def loop():
                mhz, bits = ctypes.c_uint(0), ctypes.c_ulonglong(0)
                while not self._stop.is_set():
                    if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(mhz)) == 0 and \
                            reasons_fn(h, ctypes.byref(bits)) == 0:
                        self.samples.append((float(mhz.value), int(bits.value)))
                    time.sleep(0.001)

            self._thread = threading.Thread(target=loop, daemon=True)
            self._thread.start()
            time.sleep(0.005)
            return self
        try:
            self.fh = open(self.path, "w")
            self._proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100", "-i", self.uuid or "0"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
            self.source = "nvidia-smi, 100 ms"
        except Exception:
            self._proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self._thread is not None:
            self._stop.set()
            self._thread.join()
        if self._proc is not None:
            self._proc.terminate()
            self._proc.wait()
            self.fh.close()
            try:
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                         "sw_power_cap"]
                bits = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20,
                        "hw_thermal_slowdown": 0x40}
                for r in open(self.path).read().strip().splitlines():
                    f = r.split(",")
                    self.max_mhz = float(f[2])
                    b = 0
                    for k, name in enumerate(names):
                        if f[5 + k].strip() == "Active":
                            b |= bits[name]
                    self.samples.append((float(f[1]), b))
            except Exception:
                pass

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": [],
                    "samples": 0, "source": self.source}
        reasons = set()
        for _, b in self.samples:
            for bit, name in self.REASONS.items():
                if b & bit:
                    reasons.add(name)
        return {"sm_mhz": float(np.median([m for m, _ in self.samples])),
                "sm_max_mhz": self.max_mhz, "reasons": sorted(reasons),
                "samples": len(self.samples), "source": self.source, "device": self.uuid}


class CpuSubiter:
    """The float32 C/OpenMP oracle port of one OSEM sub-iteration of the workload."""

    def __init__(self, w, threads):
        import oracle
        os.environ["OMP_NUM_THREADS"] = str(threads)
        self.o = oracle.SpectOracle(w.shape, w.dr, w.angles, [w.radius] * len(w.angles),
                                    mu=w.mu, psf=w.psf, order="ap" if w.psf else "a",
                                    precision="f32")
        self.idx = oracle.subsets(len(w.angles), w.n_subsets)[0]
        self.f = np.ones(w.shape, np.float32)
        self.g = np.ones((len(self.idx),) + w.shape[1:], np.float32) * 10
        self.nbp = np.ones(w.shape, np.float32)

    def angles(self, idx):
        """Forward, ratio, back projection and update restricted to the angles idx."""
        t0 = time.perf_counter()
        pred = self.o.forward(self.f, idx)
        bp = self.o.backward(self.g[: len(idx)] / (pred + 1e-11), idx)
        f = self.f + self.f * (1 / (self.nbp + 1e-11)) * (bp - self.nbp)
        f[f <= 0] = 0
        return time.perf_counter() - t0


def fma_cobound(w, n_sel: int, launch_ms: float, dev):
    """The PSF blur's FLOP model of the forward launch (2 P (K_r + K_z) per angle, P = the
    padded volume, full taps at every plane) against the nominal FP32 FMA peak of the device
    (SMs x 128 lanes x 2 FLOP x the maximum SM clock); None without PSF."""
    if not w.psf:
        return None
    import torch
    from pytomography_gb300 import geometry
    n, nz = w.shape[0], w.shape[2]
    lp = n + 2 * geometry.compute_pad_size(n)
    sig = geometry.psf_sigma(lp, w.radius, w.dr[0], _PsfFit(w.psf))
    k = geometry.psf_kernel_size(sig, w.dr[0], 3.0)
    flops = 2.0 * lp * lp * nz * (2 * k) * n_sel
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = 2070.0
    try:
        with open(PEAKS) as fh:
            mhz = float(json.load(fh).get("sm_max_mhz", mhz))
    except (OSError, ValueError):
        pass
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    ach = flops / (launch_ms / 1000) / 1e12
    return {"flops_per_launch": flops, "taps": k, "achieved_tflops": ach, "peak_tflops": peak,
            "frac": ach / peak, "peak_kind": f"nominal: {sms} SMs x 128 FP32 lanes x 2 FLOP x "
                                             f"{mhz:.0f} MHz"}


class _PsfFit:
    """sigma(d) = a d + b, the PSF model of the workloads (cm)."""

    def __init__(self, ab):
        self.sigma_fit_params = tuple(ab)

    @staticmethod
    def sigma_fit(d, a, b):
        return a * d + b


def osem_config(w, n_sub: int, n_sel: int, world: int) -> dict:
    """The ``config`` of an OSEM workload's line; both arms print the same one."""
    return {"workload": w.name, "subsets": n_sub, "angles_per_step": n_sel,
            "l2": "no flush; per-step working set (A 175 MB + W 175 MB + object) "
                  "exceeds the 129 MB L2" if w.shape[0] == 128 else
                  "no flush; per-step working set (A + W + object, ~60 MB) is "
                  "smaller than L2: the figure includes L2 reuse across steps",
            "parallelism": "replicas" if world > 1 else "single"}


def run_reference(args):
    """CPU implementation of the path on all host cores: each step is one angle of a
    sub-iteration (forward, ratio, back projection, update); subiter/s = 1 / (12 x t)."""
    from pytomography_gb300 import synthetic
    import oracle.build
    oracle.build.build()
    w = synthetic.config2()
    cores = len(os.sched_getaffinity(0))
    cpu = CpuSubiter(w, cores)
    n_sel = len(cpu.idx)
    times = []
    for i in range(args.warmup + args.steps):
        t = cpu.angles(cpu.idx[i % n_sel: i % n_sel + 1])
        if i >= args.warmup:
            times.append(t)
    v = 1.0 / (n_sel * float(np.mean(times)))
    line = {"metric": METRIC, "value": v, "unit": "subiter/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * n_sel * float(np.mean(times)),
            "ms_per_timed_angle": 1000 * float(np.mean(times)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": osem_config(w, w.n_subsets, n_sel, args.gpus),
            "cpu_baseline": {"value": v, "unit": "subiter/s", "cores": cores, "kind": "port",
                             "sample": f"each timed step is one angle of an OSEM sub-iteration "
                                       f"of the {w.shape[0]}^3 workload (fwd, ratio, bwd, update; "
                                       f"angles taken in turn from the first subset), float32 "
                                       f"C/OpenMP oracle; subiter/s = 1/({n_sel} x mean step "
                                       f"time)"},
            "e2e": {"value": v, "unit": "subiter/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _events_timer(fn, n, warm=3):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(n):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / n


def run_pet(args, dev):
    """TOF listmode OSEM: 200x200x96 image at 2 mm, 600 x 96 crystals (radius 400 mm),
    10M events (20% randoms), 13 TOF bins, 20 subsets of 500k events.  A step is one
    sub-iteration (TOF forward of the subset's events with the ratio epilogue, TOF back
    projection, update).  The sensitivity image is replaced by ones (one-time cost,
    excluded); the per-event additive term is the uniform randoms rate."""
    import torch
    from pytomography_gb300 import synthetic
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    w = synthetic.config3()
    H = synthetic.build_pet_system_matrix(w)
    E = w.events.shape[0]
    H.norm_BP = torch.ones(w.shape, device=dev)
    s = torch.full((E,), w.randoms_per_bin, device=dev)
    lik = PoissonLogLikelihood(H, additive_term=s)
    lik._set_n_subsets(w.n_subsets)
    f = H._get_object_initial().contiguous()
    nbps = [lik._get_normBP(k).contiguous() for k in range(w.n_subsets)]
    k_state = [0]
    if args.profile_case:
        for k in range(3):
            H.osem_step(f, lik.projections, s, nbps[k], k)
        torch.cuda.synchronize()
        print("profile case done")
        return

    def fused():
        k = k_state[0] % w.n_subsets
        H.osem_step(f, lik.projections, s, nbps[k], k)
        k_state[0] += 1

    def plain():
        k = k_state[0] % w.n_subsets
        grad = lik.compute_gradient(f, k)
        f.add_(f * (1 / (nbps[k] + 1e-11)) * grad)
        f[f <= 0] = 0
        k_state[0] += 1

    fused_ms = _events_timer(fused, args.steps)
    plain_ms = _events_timer(plain, max(10, args.steps // 5))
    sens_s = None
    if getattr(args, "pet_sensitivity", False):
        # the one-time sensitivity image over every crystal pair (C(57600, 2) = 1.66e9
        # LORs, non-TOF back projection, pairs generated on the device), timed once
        from pytomography_gb300 import _lib
        img = torch.empty(w.shape, device=dev)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        _lib.check(H._lib.gb_pet_sensitivity(H._plan, None, 0, None, None, 0.0, _lib.ptr(img),
                                             _lib.stream_handle(dev)))
        b.record()
        torch.cuda.synchronize()
        n_det = int(H.proj_meta.scanner_lut.shape[0])
        n_pairs = n_det * (n_det - 1) // 2
        sens_s = {"seconds": a.elapsed_time(b) / 1000.0, "lors": n_pairs,
                  "lors_per_s": n_pairs / (a.elapsed_time(b) / 1000.0)}
    fwd_ms = _events_timer(lambda: H.forward(f, 0), 20)
    p0 = H.forward(f, 0)
    bwd_ms = _events_timer(lambda: H.backward(p0, 0), 20)
    cpu = None
    if not args.no_cpu:
        import oracle
        from pytomography_gb300.metadata.PET import PETTOFMeta
        cores = len(os.sched_getaffinity(0))
        os.environ["OMP_NUM_THREADS"] = str(cores)
        tm = PETTOFMeta(*w.tof)
        o = oracle.PetLMOracle(w.shape, w.voxel_mm, H.proj_meta.scanner_lut.numpy(),
                               tof=(w.tof[0], float(tm.bin_width), float(tm.sigma),
                                    float(tm.center_offset), float(tm.n_sigmas)),
                               precision="f32")
        ev = w.events[0::w.n_subsets][:50000]
        img = f.cpu().numpy()
        t0 = time.perf_counter()
        pr = o.forward(img, ev)
        o.backward(1.0 / (pr + 1e-11), ev)
        t = time.perf_counter() - t0
        cpu = {"value": len(ev) / t / (E / w.n_subsets), "unit": "subiter/s", "cores": cores,
               "kind": "port", "sample": "50k events of a subset, TOF forward + back projection, "
                                         "float32 C/OpenMP oracle, scaled to 500k events"}
    line = {"metric": "PET TOF listmode OSEM subiter/s (500k events per subset)",
            "value": 1000.0 / fused_ms, "unit": "subiter/s", "n_gpus": 1, "steps": args.steps,
            "warmup": 3, "ms_per_step": fused_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "events": E, "subsets": w.n_subsets,
                       "tof_bins": w.tof[0], "image": list(w.shape)},
            "events_per_s": (E / w.n_subsets) / (fused_ms / 1000.0),
            "plain": {"value": 1000.0 / plain_ms, "ms_per_step": plain_ms},
            "forward_ms": fwd_ms, "backward_ms": bwd_ms, "cpu_baseline": cpu}
    if sens_s is not None:
        line["sensitivity_all_pairs"] = sens_s
    return line


def run_autograd(args, dev):
    """Differentiable SPECT at the 128^3 / 120-angle geometry: gradients of the Poisson NLL
    of 8 objects through the autograd Function (forward + exact adjoint over all angles),
    and fused BSREM sub-iterations with the RDP prior (beta 0.3, gamma 2)."""
    import torch
    from pytomography_gb300 import synthetic
    from pytomography_gb300.algorithms import BSREM
    from pytomography_gb300.autograd import poisson_nll
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    from pytomography_gb300.priors import RelativeDifferencePrior
    ws = [synthetic.config2(seed=10 + i) for i in range(8)]
    H = synthetic.build_system_matrix(ws[0])
    gs = torch.stack([synthetic.poisson_projections(H, w).to(dev) for w in ws])
    fb = torch.ones((8, *ws[0].shape), device=dev, requires_grad=True)

    def grad_step():
        fb.grad = None
        poisson_nll(fb, H, gs).backward()

    grad_ms = _events_timer(grad_step, max(3, args.steps // 20))
    lik = PoissonLogLikelihood(H, gs[0])
    alg = BSREM(lik, prior=RelativeDifferencePrior(beta=0.3, gamma=2))
    alg(1, 10)  # warm-up, plans and normalisation
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_it = 2
    alg(n_it, 10)
    torch.cuda.synchronize()
    bsrem_ms = (time.perf_counter() - t0) * 1000.0 / (n_it * 10)
    line = {"metric": "Poisson-NLL object gradients/s (128^3, 120 angles, att+PSF)",
            "value": 8 * 1000.0 / grad_ms, "unit": "gradients/s", "n_gpus": 1,
            "steps": max(3, args.steps // 20), "warmup": 3, "ms_per_step": grad_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "8 objects x 128^3, 120 angles, att+PSF, autograd",
                       "bsrem": "RDP beta 0.3 gamma 2, 10 subsets"},
            "bsrem": {"value": 1000.0 / bsrem_ms, "unit": "subiter/s", "ms_per_step": bsrem_ms}}
    return line


def run_serving(args, dev):
    """32 uneven reconstructions (sizes 64/96/128^3, 60/90/120 angles, att + PSF, 10
    subsets): sub-iterations summed over reconstructions per second, batched (one
    persistent launch per phase across all 32, replayed from CUDA graphs) vs plain (each
    reconstruction in turn through the per-call path)."""
    import torch
    from pytomography_gb300 import synthetic
    from pytomography_gb300.batched import BatchedOSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    ws = synthetic.config5()
    Hs = [synthetic.build_system_matrix(w) for w in ws]
    gs = [synthetic.poisson_projections(H, w).to(dev) for H, w in zip(Hs, ws)]
    R = len(ws)
    if args.profile_case:  # three batched sub-iterations, no graphs (for ncu)
        b = BatchedOSEM([PoissonLogLikelihood(H, g) for H, g in zip(Hs, gs)], n_subsets=10,
                        use_graphs=False)
        for k in range(3):
            b.step(k)
        torch.cuda.synchronize()
        print("profile case done")
        return {}
    # plain: each reconstruction's sub-iterations through forward / torch / backward / torch
    liks = [PoissonLogLikelihood(H, g) for H, g in zip(Hs, gs)]
    for lik in liks:
        lik._set_n_subsets(10)
    fs = [torch.ones(w.shape, device=dev) for w in ws]

    def plain_round(k):
        for lik, f in zip(liks, fs):
            grad = lik.compute_gradient(f, k)
            nb = lik._get_normBP(k)
            f.add_(f * (1 / (nb + 1e-11)) * grad)
            f[f <= 0] = 0

    for k in range(3):
        plain_round(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n_plain = 10
    e0.record()
    for k in range(n_plain):
        plain_round(k % 10)
    e1.record()
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / n_plain
    # the reference's per-call GPU sequence in plain PyTorch: one round over all
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from torch_reference import TorchReferenceProjector
    refs = [TorchReferenceProjector(H) for H in Hs]
    tr = [torch.ones(w.shape, device=dev) for w in ws]
    tr[0] = refs[0].osem_subiteration(tr[0], gs[0], None, liks[0]._get_normBP(0), 0)
    torch.cuda.synchronize()
    e0.record()
    for i in range(R):
        tr[i] = refs[i].osem_subiteration(tr[i], gs[i], None, liks[i]._get_normBP(1), 1)
    e1.record()
    torch.cuda.synchronize()
    torch_ref_ms = e0.elapsed_time(e1)
    del refs, tr
    batch = BatchedOSEM([PoissonLogLikelihood(H, g) for H, g in zip(Hs, gs)], n_subsets=10)
    batch.capture()
    for k in range(max(3, args.warmup)):
        batch.step(k % 10)
    torch.cuda.synchronize()
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b0.record()
    for k in range(args.steps):
        batch.step(k % 10)
    b1.record()
    torch.cuda.synchronize()
    batch_ms = b0.elapsed_time(b1) / args.steps
    line = {"metric": "OSEM subiter/s summed over 32 uneven reconstructions (att+PSF)",
            "value": R * 1000.0 / batch_ms, "unit": "subiter/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": batch_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "serving: 32 reconstructions, sizes 64/96/128^3, "
                                   "60/90/120 angles, att+PSF, 10 subsets",
                       "sizes": [w.shape[0] for w in ws],
                       "angles": [len(w.angles) for w in ws]},
            "plain": {"value": R * 1000.0 / plain_ms, "ms_per_step": plain_ms},
            "batched_vs_plain": plain_ms / batch_ms,
            "torch_reference": {"value": R * 1000.0 / torch_ref_ms, "ms_per_step": torch_ref_ms,
                                "what": "the reference's per-call GPU sequence restated in "
                                        "plain PyTorch float32, one round of 32"},
            "batched_vs_torch_reference": torch_ref_ms / batch_ms}
    return line


def run_osem(args, dev, w, rank, world, dist, full=True):
    """One OSEM workload: fused sub-iterations from graphs (the line's value), the plain
    per-call path, the PyTorch restatement of the reference sequence, the forward
    projector's roofline, end to end through the public API and (full) the CPU baselines."""
    import torch
    from pytomography_gb300 import _lib, synthetic
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood
    metric = METRIC if w.shape[0] == 128 else "OSEM subiter/s at 64^3x64 ang (att)"
    H = synthetic.build_system_matrix(w)
    g_host = synthetic.poisson_projections(H, w)
    g = g_host.to(dev)
    lik = PoissonLogLikelihood(H, g)
    lik._set_n_subsets(w.n_subsets)
    nbps = [nb.contiguous() for nb in lik.norm_BPs]
    f = torch.ones(w.shape, device=dev)
    n_sub = w.n_subsets
    n_sel = len(w.angles) // n_sub  # angles per sub-iteration (equal subsets here)
    if args.profile_case:
        for k in range(3):
            H.osem_step(f, g, None, nbps[k], k)
        torch.cuda.synchronize()
        print("profile case done")
        return None

    # ---- plain per-call path (reference sequence through the drop-in projector)
    def plain_step(k):
        grad = lik.compute_gradient(f, k)
        pre = f * (1 / (nbps[k] + 1e-11))
        f.add_(pre * grad)
        f[f <= 0] = 0

    for k in range(args.warmup):
        plain_step(k % n_sub)
    torch.cuda.synchronize()
    n_plain = max(n_sub, min(args.steps, 50))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(n_plain):
        plain_step(k % n_sub)
    e1.record()
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / n_plain

    # ---- the reference's per-call GPU sequence in plain PyTorch (context line)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from torch_reference import TorchReferenceProjector
    R = TorchReferenceProjector(H)
    ft = torch.ones(w.shape, device=dev)
    for k in range(2):
        ft = R.osem_subiteration(ft, g, None, nbps[k], k)
    torch.cuda.synchronize()
    n_tr = 5
    e0.record()
    for k in range(n_tr):
        ft = R.osem_subiteration(ft, g, None, nbps[k % n_sub], k % n_sub)
    e1.record()
    torch.cuda.synchronize()
    torch_ref_ms = e0.elapsed_time(e1) / n_tr
    del R, ft

    # ---- fused sub-iterations, one CUDA graph per subset
    f.fill_(1.0)
    pred = torch.empty((n_sel, *w.shape[1:]), device=dev)
    stream = torch.cuda.Stream(device=dev)
    graphs = []
    with torch.cuda.stream(stream):
        for k in range(n_sub):  # warm the plan on this stream before capture
            H.osem_step(f, g, None, nbps[k], k, predicted=pred)
    torch.cuda.synchronize()
    for k in range(n_sub):
        gr = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gr, stream=stream):
            H.osem_step(f, g, None, nbps[k], k, predicted=pred)
        graphs.append(gr)
    f.fill_(1.0)
    torch.cuda.synchronize()
    for k in range(args.warmup):
        graphs[k % n_sub].replay()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = Clocks(os.path.join(args.out, "clocks.csv"), dev) if rank == 0 else None
    os.makedirs(args.out, exist_ok=True)
    if clocks:
        clocks.__enter__()
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cur = torch.cuda.current_stream()
    s0.record(cur)
    for k in range(args.steps):
        graphs[k % n_sub].replay()
    s1.record(cur)
    torch.cuda.synchronize()
    if clocks:
        clocks.__exit__()
    ms = max_over_ranks(s0.elapsed_time(s1), dist, dev)
    fused_ms = ms / args.steps
    value = world * args.steps / (ms / 1000.0)

    # ---- roofline of the forward projector (kernels launched on `cur`)
    fwd_bytes, bwd_bytes, sub_bytes = alg_bytes_subiter(w.shape[0], n_sel, 1)
    proj = torch.empty((n_sel, *w.shape[1:]), device=dev)
    obj = torch.empty(w.shape, device=dev)
    for _ in range(3):
        lib = H._lib
        lib.gb_spect_forward(H._plan, _lib.ptr(f), _lib.ptr(proj), 0, _lib.stream_handle(dev))
    reps = 20
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(cur)
    for r in range(reps):
        _lib.check(H._lib.gb_spect_forward(H._plan, _lib.ptr(f), _lib.ptr(proj), r % n_sub,
                                           _lib.stream_handle(dev)))
    a1.record(cur)
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b0.record(cur)
    for r in range(reps):
        _lib.check(H._lib.gb_spect_backward(H._plan, _lib.ptr(proj), _lib.ptr(obj), r % n_sub, 0,
                                            _lib.stream_handle(dev)))
    b1.record(cur)
    torch.cuda.synchronize()
    fwd_ms = a0.elapsed_time(a1) / reps
    bwd_ms = b0.elapsed_time(b1) / reps
    hbm, peak_kind = peaks()
    ach = fwd_bytes / (fwd_ms / 1000) / 1e9

    # ---- end to end through the public API from host tensors
    mu_host = torch.tensor(w.mu, dtype=torch.float32).pin_memory()
    g_pin = g_host.pin_memory()
    n_e2e = 2
    out_host = torch.empty(w.shape, pin_memory=True)
    e2e_times = []
    for rep in range(n_e2e + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w.mu = mu_host
        H2 = synthetic.build_system_matrix(w)
        lik2 = PoissonLogLikelihood(H2, g_pin.to(dev, non_blocking=True))
        rec = OSEM(lik2)(w.n_iters, w.n_subsets)
        out_host.copy_(rec)
        torch.cuda.synchronize()
        if rep > 0:
            e2e_times.append(time.perf_counter() - t0)
        del H2, lik2, rec
    e2e_subiter = w.n_iters * w.n_subsets / float(np.mean(e2e_times))

    cpu = None
    cpu_torch = None
    if rank == 0 and not args.no_cpu:
        cores = len(os.sched_getaffinity(0))
        c = CpuSubiter(w, cores)
        t = c.angles(c.idx)
        cpu = {"value": 1.0 / t, "unit": "subiter/s", "cores": cores, "kind": "port",
               "sample": f"one OSEM sub-iteration ({n_sel} angles fwd+ratio+bwd+update) of "
                         f"the {w.shape[0]}^3 workload, float32 C/OpenMP oracle"}
        # the reference's per-call PyTorch sequence on the host cores: two angles of the
        # first subset forward + back projected, scaled to the 12-angle sub-iteration
        torch.set_num_threads(cores)
        Rc = TorchReferenceProjector(H, device="cpu")
        two = [int(i) for i in H.subset_indices_array[0][:2].tolist()]
        fc = torch.ones(w.shape)
        Rc.forward(fc, two[:1])
        t0 = time.perf_counter()
        pc = Rc.forward(fc, two)
        Rc.backward(torch.ones_like(pc), two)
        t_two = time.perf_counter() - t0
        cpu_torch = {"value": 2.0 / (t_two * n_sel), "unit": "subiter/s", "cores": cores,
                     "kind": "port", "sample": "the reference's per-call PyTorch sequence "
                     "(tests/torch_reference.py) on torch CPU with all host threads: 2 "
                     f"angles forward + back projected, scaled to {n_sel}"}
        del Rc

    line = None
    if rank == 0:
        line = {
            "metric": metric, "value": value, "unit": "subiter/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": fused_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": osem_config(w, n_sub, n_sel, world),
            "plain": {"value": 1000.0 / plain_ms, "unit": "subiter/s", "ms_per_step": plain_ms},
            "fused_vs_plain": plain_ms / fused_ms,
            "torch_reference": {"value": 1000.0 / torch_ref_ms, "unit": "subiter/s",
                                "ms_per_step": torch_ref_ms,
                                "what": "the reference's per-call GPU sequence restated in "
                                        "plain PyTorch float32 (tests/torch_reference.py)"},
            "fused_vs_torch_reference": torch_ref_ms / fused_ms,
            "e2e": {"value": e2e_subiter, "unit": "subiter/s",
                    "h2d_bytes_per_step": int((g_host.numel() + mu_host.numel()) * 4
                                              / (w.n_iters * w.n_subsets)),
                    "d2h_bytes_per_step": int(out_host.numel() * 4 / (w.n_iters * w.n_subsets)),
                    "what": "OSEM(4,10) from host tensors incl. plan build and normalisation"},
            "roofline": {"bound": "hbm", "kernel": "forward projector (k_fwd_psf + k_reduce)"
                         if w.psf else "forward projector (k_fwd_nopsf + k_reduce)",
                         "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                         "peak_kind": peak_kind,
                         "traffic": FWD_DRAM_BYTES_PER_LAUNCH if w.shape[0] == 128 else None,
                         "traffic_source": "constant from a separate ncu capture of one "
                                           "launch (dram__bytes_read.sum + "
                                           "dram__bytes_write.sum); not measured by this run",
                         "alg_bytes_per_launch": fwd_bytes, "launch_ms": fwd_ms,
                         "fma_cobound": fma_cobound(w, n_sel, fwd_ms, dev)},
            "backward_ms": bwd_ms,
            "alg_gbs_per_subiter": sub_bytes / (fused_ms / 1000) / 1e9,
            "gpu_launches": 4 * args.steps,
            "clocks": clocks.summary() if clocks else None,
            "cpu_baseline": cpu,
            "cpu_torch_reference": cpu_torch,
        }
    return line




def extra_configs(args, dev):
    """The other benchmark configurations, each timed on its own with CUDA events and
    reported beside the headline: 64^3 x 64 OSEM, PET TOF listmode OSEM (10M events) with
    the one-time all-pairs sensitivity image, Poisson-NLL gradients of 8 objects and BSREM,
    and the 32-reconstruction serving batch."""
    from pytomography_gb300 import synthetic
    import argparse as _ap
    sub = _ap.Namespace(**vars(args))
    sub.steps, sub.warmup, sub.no_cpu, sub.profile_case = min(args.steps, 50), 3, True, False
    out = {}

    def keep(line, keys):
        return {k: line[k] for k in keys if k in line}

    t0 = time.perf_counter()
    l1 = run_osem(sub, dev, synthetic.config1(), 0, 1, None, full=False)
    out["osem64"] = keep(l1, ("metric", "value", "unit", "ms_per_step", "plain", "fused_vs_plain",
                              "e2e", "roofline", "config"))
    sub.pet_sensitivity = True  # the one-time all-pairs sensitivity image, timed once
    l3 = run_pet(sub, dev)
    out["pet"] = keep(l3, ("metric", "value", "unit", "ms_per_step", "events_per_s", "plain",
                           "forward_ms", "backward_ms", "sensitivity_all_pairs", "config"))
    l4 = run_autograd(sub, dev)
    out["autograd"] = keep(l4, ("metric", "value", "unit", "ms_per_step", "bsrem", "config"))
    l5 = run_serving(sub, dev)
    out["serving"] = keep(l5, ("metric", "value", "unit", "ms_per_step", "plain",
                               "batched_vs_plain", "config"))
    out["wall_s"] = time.perf_counter() - t0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gbtomo", choices=["gbtomo", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--out", default=os.path.join(ROOT, "bench_out"),
                    help="folder for the clock samples of the timed region (clocks.csv)")
    ap.add_argument("--headline-only", action="store_true",
                    help="report only the 128^3 workload (skip the other configurations)")
    ap.add_argument("--pet-sensitivity", action="store_true",
                    help="with --workload pet: also time the all-pairs sensitivity image once")
    ap.add_argument("--profile-forward", type=int, default=0, choices=[0, 1, 2],
                    help="run three 12-angle forward projections of the 128^3 workload with "
                         "forward variant 1 or 2 and exit (for ncu)")
    ap.add_argument("--profile-case", action="store_true",
                    help="run 3 fused sub-iterations of the workload and exit (for ncu)")
    ap.add_argument("--workload", default="osem128",  # osem64: the 64^3 / 64-angle att case
                    choices=["osem128", "osem64", "serving", "pet", "autograd"],
                    help="osem128: the 128^3 x 120-angle reconstruction (default); serving: "
                         "32 uneven reconstructions, batched vs plain; pet: TOF listmode OSEM "
                         "(10M events); autograd: Poisson-NLL gradients of 8 objects + BSREM")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.warmup < 3:
        args.warmup = 3

    import torch
    from pytomography_gb300 import _lib, synthetic
    from pytomography_gb300.algorithms import OSEM
    from pytomography_gb300.likelihoods import PoissonLogLikelihood

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    _lib.load()

    if args.profile_forward:
        w = synthetic.config2()
        H = synthetic.build_system_matrix(w)
        H.set_n_subsets(w.n_subsets)
        H.set_tuning(fwd_variant=args.profile_forward)
        f = torch.tensor(w.activity, dtype=torch.float32, device=dev)
        for k in range(3):
            H.forward(f, k)
        torch.cuda.synchronize()
        print("profile forward done", args.profile_forward)
        return
    if args.workload == "serving":
        line = run_serving(args, dev)
        if not args.profile_case:
            print(json.dumps(line))
        return
    if args.workload == "pet":
        print(json.dumps(run_pet(args, dev)))
        return
    if args.workload == "autograd":
        print(json.dumps(run_autograd(args, dev)))
        return
    w = synthetic.config1() if args.workload == "osem64" else synthetic.config2()
    line = run_osem(args, dev, w, rank, world, dist, full=True)
    if args.profile_case:
        return
    if rank == 0 and world == 1 and args.workload == "osem128" and not args.headline_only:
        line["configs"] = extra_configs(args, dev)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
