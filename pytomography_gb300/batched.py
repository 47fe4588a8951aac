"""Batched OSEM over many independent SPECT reconstructions.

Each reconstruction keeps its own ``SPECTSystemMatrix`` (its own geometry, angle count,
PSF table and attenuation factors).  Two execution forms:

* ``mode="persistent"`` (default): one C batch (``gb_spect_batch_create``) over all the
  reconstructions' plans.  A sub-iteration of every reconstruction is four kernel
  launches in all: a persistent forward projector that dequeues the work items of every
  reconstruction from one list ordered by estimated cost (largest first), one reduction
  with the likelihood-ratio epilogue, a persistent rotated-frame back-projection pass and
  one gather with the OSEM update.  The plans are given a common PSF tap bucket first
  (zero taps added; the projections are unchanged).  Batches hold up to 32
  reconstructions; larger sets are split into several batches.
* ``mode="streams"``: each reconstruction's fused sub-iteration launched on its own
  plan, round-robin over several streams.

With ``use_graphs`` every subset index's sub-iterations are recorded once into a CUDA
graph and replayed.  The reference runs each reconstruction's OSEM loop in turn
(algorithms/preconditioned_gradient_ascent.py:80-129 over
projectors/SPECT/spect_system_matrix.py:120-201).

Usage::

    batch = BatchedOSEM([PoissonLogLikelihood(H_i, g_i) for i in ...], n_subsets=10)
    recons = batch(n_iters=4)
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .likelihoods import PoissonLogLikelihood
from .projectors.SPECT import SPECTSystemMatrix

MAX_BATCH = 32


def _ptr_array(tensors):
    arr = (ctypes.c_void_p * len(tensors))()
    for i, t in enumerate(tensors):
        arr[i] = None if t is None else t.data_ptr()
    return arr


class SpectBatch:
    """A C batch over plans (reconstructions, or objects sharing one plan): forward and
    back projection of every entry in one launch per phase."""

    def __init__(self, system_matrices) -> None:
        sms = list(system_matrices)
        if not 1 <= len(sms) <= MAX_BATCH:
            raise ValueError(f"a batch holds 1 to {MAX_BATCH} entries")
        self.sms = sms
        self._lib = sms[0]._lib
        self.device = sms[0].device
        plans = (ctypes.c_void_p * len(sms))(*[sm._plan.value for sm in sms])
        h = ctypes.c_void_p()
        _lib.check(self._lib.gb_spect_batch_create(plans, len(sms), ctypes.byref(h)))
        self._h = h
        self._keep = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None:
            try:
                self._lib.gb_spect_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    @staticmethod
    def _code(subset_idx) -> int:
        return -1 if subset_idx is None else int(subset_idx)

    def forward(self, objects, subset_idx=None, out=None):
        """Projections of every entry's object; ``out`` (optional) is a list of output
        tensors or one stacked tensor whose slices receive them."""
        if out is None:
            out = [torch.empty((sm._n_sel(subset_idx), *sm.proj_meta.shape[1:]),
                               device=self.device, dtype=torch.float32) for sm in self.sms]
        outs = list(out)
        objs = [o.contiguous() for o in objects]
        _lib.check(self._lib.gb_spect_batch_forward(
            self._h, _ptr_array(objs), _ptr_array(outs), self._code(subset_idx),
            _lib.stream_handle(self.device)))
        return out

    def backward(self, projs, subset_idx=None, adjoint: bool = False, out=None):
        if out is None:
            out = [torch.empty(tuple(sm.object_meta.shape), device=self.device,
                               dtype=torch.float32) for sm in self.sms]
        outs = list(out)
        ps = [p.contiguous() for p in projs]
        _lib.check(self._lib.gb_spect_batch_backward(
            self._h, _ptr_array(ps), _ptr_array(outs), self._code(subset_idx), int(adjoint),
            _lib.stream_handle(self.device)))
        return out

    def osem_step(self, objects, projections, additive, norm_bps, subset_idx) -> None:
        _lib.check(self._lib.gb_spect_batch_osem_step(
            self._h, _ptr_array(objects), _ptr_array(projections),
            None if additive is None else _ptr_array(additive), _ptr_array(norm_bps),
            self._code(subset_idx), _lib.stream_handle(self.device)))


def common_psf_bucket(system_matrices) -> None:
    """Rebuild plans so that all share the largest PSF tap bucket among them."""
    k = max(sm.psf_bucket for sm in system_matrices)
    for sm in system_matrices:
        if sm.psf_bucket != k:
            sm._rebuild_plan(k)


class BatchedOSEM:
    def __init__(self, likelihoods, n_subsets: int, object_initial=None, n_streams: int = 4,
                 use_graphs: bool = True, autotune: bool = True,
                 mode: str = "persistent") -> None:
        if not likelihoods:
            raise ValueError("no reconstructions")
        for lik in likelihoods:
            if type(lik) is not PoissonLogLikelihood or \
                    not isinstance(lik.system_matrix, SPECTSystemMatrix):
                raise NotImplementedError("batched OSEM needs PoissonLogLikelihood over "
                                          "SPECTSystemMatrix")
        if mode not in ("persistent", "streams"):
            raise ValueError("mode is 'persistent' or 'streams'")
        self.likelihoods = list(likelihoods)
        self.n_subsets = int(n_subsets)
        self.use_graphs = use_graphs
        self.device = self.likelihoods[0].system_matrix.device
        sms = [lik.system_matrix for lik in self.likelihoods]
        if mode == "persistent" and not all(self._batchable(sm) for sm in sms):
            mode = "streams"
        self.mode = mode
        if mode == "persistent":
            common_psf_bucket(sms)
        self.objects = []
        for i, lik in enumerate(self.likelihoods):
            sm = lik.system_matrix
            if object_initial is not None:
                f = object_initial[i].to(sm.device, torch.float32).contiguous().clone()
            else:
                f = sm._get_object_initial(sm.device).to(torch.float32).contiguous()
            self.objects.append(f)
            lik._set_n_subsets(self.n_subsets)
            if autotune and mode == "streams":  # tile shapes per geometry, once per process
                sm.autotune(0 if self.n_subsets > 1 else None)
            lik.projections = lik.projections.to(sm.device, torch.float32).contiguous()
        if mode == "persistent":
            self._batches = []
            for i0 in range(0, len(sms), MAX_BATCH):
                self._batches.append((i0, SpectBatch(sms[i0:i0 + MAX_BATCH])))
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(max(1, n_streams))]
        self._graphs = None

    @staticmethod
    def _batchable(sm) -> bool:
        nx, _, nz = (int(v) for v in sm.object_meta.shape)
        return "p" in sm._order and nx <= 128 and nz <= 128 and nz % 4 == 0 and not sm._no_pad

    @property
    def n_reconstructions(self) -> int:
        return len(self.likelihoods)

    def _subset_idx(self, k: int):
        return None if self.n_subsets == 1 else k

    def _issue(self, k: int) -> None:
        sub = self._subset_idx(k)
        if self.mode == "persistent":
            for i0, b in self._batches:
                liks = self.likelihoods[i0:i0 + len(b.sms)]
                add = [lik.additive_term if lik.exists_additive_term else None for lik in liks]
                b.osem_step(self.objects[i0:i0 + len(b.sms)], [lik.projections for lik in liks],
                            add if any(a is not None for a in add) else None,
                            [lik._get_normBP(sub).contiguous() for lik in liks], sub)
            return
        # all reconstructions' sub-iteration k, round-robin over the streams
        main = torch.cuda.current_stream(self.device)
        for s in self.streams:
            s.wait_stream(main)
        for i, lik in enumerate(self.likelihoods):
            st = self.streams[i % len(self.streams)]
            with torch.cuda.stream(st):
                sm = lik.system_matrix
                s_add = lik.additive_term if lik.exists_additive_term else None
                sm.osem_step(self.objects[i], lik.projections, s_add, lik._get_normBP(sub), sub)
        for s in self.streams:
            main.wait_stream(s)

    def capture(self) -> None:
        """Record one CUDA graph per subset index (call before timing)."""
        # one eager pass of every subset warms the plans (and the capture streams)
        saved = [f.clone() for f in self.objects]
        for k in range(self.n_subsets):
            self._issue(k)
        torch.cuda.synchronize(self.device)
        for f, s in zip(self.objects, saved):
            f.copy_(s)
        graphs = []
        cap = torch.cuda.Stream(device=self.device)
        for k in range(self.n_subsets):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=cap):
                self._issue(k)
            graphs.append(g)
        torch.cuda.synchronize(self.device)
        self._graphs = graphs

    def step(self, k: int) -> None:
        if self.use_graphs:
            if self._graphs is None:
                self.capture()
            self._graphs[k].replay()
        else:
            self._issue(k)

    def __call__(self, n_iters: int):
        for _ in range(n_iters):
            for k in range(self.n_subsets):
                self.step(k)
        return self.objects


def plain_osem(likelihoods, n_iters: int, n_subsets: int):
    """The per-call drop-in path: each reconstruction in turn, forward / ratio / backward /
    update as separate calls (what the reference's OSEM loop does with this projector)."""
    from .algorithms import OSEM
    return [OSEM(lik, fused=False)(n_iters, n_subsets) for lik in likelihoods]
