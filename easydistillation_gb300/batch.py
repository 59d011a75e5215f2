"""Batched, CUDA-graph-captured elemental runs.

Many timeslices (and several lattice volumes with different Ne) are served by
batched plans: every batch is ONE pass of the library's kernels (chains of
all timeslices, one pair-contraction launch for all of them, one combine per
timeslice).  The pass is allocation-free and stream-ordered, so it is
captured once in a CUDA graph and replayed for every batch; inputs go
through static device buffers.  Batches are admitted by HBM footprint: a
volume's batch size is the largest whose plan workspace (plus the static
buffers) fits the free device memory.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Sequence

import torch

from .insertion import num_derivative
from .ops import ElementalPlan


def admit_batch(latt_size, Ne, num_nabla, momentum_list, precision="fp64", device=None, max_batch=8,
                reserve=0.1, static_buffers=True) -> int:
    """Largest batch (1..max_batch) whose plan workspace, plus the static
    input/output buffers of a graphed batch, fits the free HBM of ``device``
    while keeping a ``reserve`` fraction free."""
    device = torch.device(device or "cuda")
    free, _total = torch.cuda.mem_get_info(device)
    budget = free * (1.0 - reserve)
    Lx, Ly, Lz, Lt = latt_size
    V3 = Lx * Ly * Lz
    per_t_static = (Ne * V3 * 3 * 16 + 3 * V3 * 9 * 16 +
                    num_derivative(num_nabla) * len(momentum_list) * Ne * Ne * 16) if static_buffers else 0
    best = 1
    for b in range(1, max_batch + 1):
        need = ElementalPlan(latt_size, Ne, num_nabla, momentum_list, precision, device, batch=b).workspace_bytes
        if need + b * per_t_static <= budget:
            best = b
        else:
            break
    return best


class GraphedElementalBatch:
    """One batched plan plus static buffers and a captured CUDA graph.

    ``run(links, evecs)`` copies up to ``batch`` timeslices of inputs
    (``links[b]``: complex128 ``[3, Lz, Ly, Lx, 3, 3]`` spatial links,
    ``evecs[b]``: ``[Ne, V3*3]`` c128/c64 reference-layout vectors) into the
    static buffers, replays the graph and returns the static output
    ``[batch, Nderiv, Nmom, Ne, Ne]`` (valid for the first len(links) rows)."""

    def __init__(self, latt_size, Ne, num_nabla, momentum_list, precision="f16x3", batch=None, device=None,
                 evec_dtype=torch.complex128):
        self.device = torch.device(device or "cuda")
        self.latt_size = list(latt_size)
        Lx, Ly, Lz, Lt = latt_size
        self.V3 = Lx * Ly * Lz
        self.Ne = Ne
        if batch is None:
            batch = admit_batch(latt_size, Ne, num_nabla, momentum_list, precision, self.device)
        self.batch = batch
        self.plan = ElementalPlan(latt_size, Ne, num_nabla, momentum_list, precision, self.device, batch=batch)
        nd, nm = num_derivative(num_nabla), len(momentum_list)
        self.links = torch.zeros((batch, 3, Lz, Ly, Lx, 3, 3), dtype=torch.complex128, device=self.device)
        eye = torch.eye(3, dtype=torch.complex128, device=self.device)
        self.links[...] = eye  # valid SU(3) links until real ones are copied in
        self.evecs = torch.zeros((batch, Ne, self.V3 * 3), dtype=evec_dtype, device=self.device)
        self.out = torch.empty((batch, nd, nm, Ne, Ne), dtype=torch.complex128, device=self.device)
        self.graph = None
        self._n = None

    def _launch(self, n):
        self.plan.run_batch([self.links[b] for b in range(n)], self.V3 * 9, 9, [self.evecs[b] for b in range(n)],
                            [self.out[b] for b in range(n)])

    def capture(self, n=None):
        n = n or self.batch
        self._launch(n)  # warm-up outside the capture (function attributes, first-use setup)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self._launch(n)
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph, self._n = g, n
        return g

    def run(self, links: Sequence[torch.Tensor], evecs: Sequence[torch.Tensor]):
        n = len(links)
        if n != len(evecs) or not (0 < n <= self.batch):
            raise ValueError(f"need 1..{self.batch} timeslices")
        for b in range(n):
            self.links[b].copy_(links[b], non_blocking=True)
            self.evecs[b].copy_(evecs[b].reshape(self.Ne, -1), non_blocking=True)
        if self.graph is None or self._n != n:
            self.capture(n)
        self.graph.replay()
        return self.out[:n]


@dataclass
class VolumeGroup:
    latt_size: List[int]
    Ne: int
    timeslices: List[int]


def run_mixed_volumes(groups: Dict[str, VolumeGroup], links: Dict[str, torch.Tensor],
                      evecs: Dict[str, torch.Tensor], num_nabla, momentum_list, precision="f16x3",
                      max_batch=8, device=None):
    """Elementals for several lattice volumes (each with its own Ne): each
    volume gets a graphed batch sized by HBM admission; its timeslices are
    processed batch by batch.  ``links[name]``: ``[3, Lt, Lz, Ly, Lx, 3, 3]``;
    ``evecs[name]``: ``[Lt, Ne, V3*3]``.  Returns {name: [n_t, Nderiv, Nmom, Ne, Ne]}."""
    out = {}
    for name, g in groups.items():
        runner = GraphedElementalBatch(g.latt_size, g.Ne, num_nabla, momentum_list, precision,
                                       batch=min(max_batch, admit_batch(g.latt_size, g.Ne, num_nabla, momentum_list,
                                                                        precision, device, max_batch)),
                                       device=device)
        res = []
        ts = list(g.timeslices)
        for s0 in range(0, len(ts), runner.batch):
            chunk = ts[s0 : s0 + runner.batch]
            r = runner.run([links[name][:, t] for t in chunk], [evecs[name][t] for t in chunk])
            res.append(r.clone())
        out[name] = torch.cat(res)
        if precision != "fp64":
            runner.plan.check_status()
        del runner
    return out
