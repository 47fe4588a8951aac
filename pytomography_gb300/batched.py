"""Batched OSEM over many independent SPECT reconstructions.

Each reconstruction keeps its own ``SPECTSystemMatrix`` plan (its own geometry, angle
count, PSF table and attenuation factors).  For every subset index ``k`` the fused
sub-iterations of all reconstructions are recorded once into a CUDA graph and the
graphs are replayed for every iteration; inside a graph the reconstructions are spread
over several streams so that their kernels run concurrently and small problems fill the
GPU together.  Each plan's kernel tiles are picked by the autotuner (timed once per
geometry and process).  The plain alternative runs the same reconstructions one after another
through the per-call drop-in path.

Usage::

    batch = BatchedOSEM([PoissonLogLikelihood(H_i, g_i) for i in ...], n_subsets=10)
    recons = batch(n_iters=4)
"""
from __future__ import annotations

import torch

from .likelihoods import PoissonLogLikelihood
from .projectors.SPECT import SPECTSystemMatrix


class BatchedOSEM:
    def __init__(self, likelihoods, n_subsets: int, object_initial=None, n_streams: int = 4,
                 use_graphs: bool = True, autotune: bool = True) -> None:
        if not likelihoods:
            raise ValueError("no reconstructions")
        for lik in likelihoods:
            if type(lik) is not PoissonLogLikelihood or \
                    not isinstance(lik.system_matrix, SPECTSystemMatrix):
                raise NotImplementedError("batched OSEM needs PoissonLogLikelihood over "
                                          "SPECTSystemMatrix")
        self.likelihoods = list(likelihoods)
        self.n_subsets = int(n_subsets)
        self.use_graphs = use_graphs
        self.device = self.likelihoods[0].system_matrix.device
        self.objects = []
        for i, lik in enumerate(self.likelihoods):
            sm = lik.system_matrix
            if object_initial is not None:
                f = object_initial[i].to(sm.device, torch.float32).contiguous().clone()
            else:
                f = sm._get_object_initial(sm.device).to(torch.float32).contiguous()
            self.objects.append(f)
            lik._set_n_subsets(self.n_subsets)
            if autotune:  # tile shapes per geometry, timed once per process
                sm.autotune(0 if self.n_subsets > 1 else None)
            lik.projections = lik.projections.to(sm.device, torch.float32).contiguous()
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(max(1, n_streams))]
        self._graphs = None

    @property
    def n_reconstructions(self) -> int:
        return len(self.likelihoods)

    def _subset_idx(self, k: int):
        return None if self.n_subsets == 1 else k

    def _issue(self, k: int) -> None:
        """All reconstructions' sub-iteration k, round-robin over the streams."""
        main = torch.cuda.current_stream(self.device)
        for s in self.streams:
            s.wait_stream(main)
        for i, lik in enumerate(self.likelihoods):
            st = self.streams[i % len(self.streams)]
            with torch.cuda.stream(st):
                sm = lik.system_matrix
                s_add = lik.additive_term if lik.exists_additive_term else None
                sm.osem_step(self.objects[i], lik.projections, s_add,
                             lik._get_normBP(self._subset_idx(k)), self._subset_idx(k))
        for s in self.streams:
            main.wait_stream(s)

    def capture(self) -> None:
        """Record one CUDA graph per subset index (call before timing)."""
        # one eager pass of every subset on the capture streams warms the plans
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
