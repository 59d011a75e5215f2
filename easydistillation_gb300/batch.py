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
from .ops import ElementalPlan, gemm_multi


def admit_batch(latt_size, Ne, num_nabla, momentum_list, precision="fp64", device=None, max_batch=8,
                reserve=0.1, static_buffers=True, forms=(True,)) -> int:
    """Largest batch (1..max_batch) whose plan workspace, plus the static
    input/output buffers of a graphed batch, fits the free HBM of ``device``
    while keeping a ``reserve`` fraction free; with several GEMM ``forms``
    (``factorise`` values) the largest of their workspaces."""
    device = torch.device(device or "cuda")
    free, _total = torch.cuda.mem_get_info(device)
    budget = free * (1.0 - reserve)
    Lx, Ly, Lz, Lt = latt_size
    V3 = Lx * Ly * Lz
    per_t_static = (Ne * V3 * 3 * 16 + 3 * V3 * 9 * 16 +
                    num_derivative(num_nabla) * len(momentum_list) * Ne * Ne * 16) if static_buffers else 0
    best = 1
    for b in range(1, max_batch + 1):
        need = 0
        for f in forms:
            try:
                need = max(need, ElementalPlan(latt_size, Ne, num_nabla, momentum_list, precision, device, batch=b,
                                               factorise=f).workspace_bytes)
            except ValueError:  # a form this mode does not take
                pass
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
    ``[batch, Nderiv, Nmom, Ne, Ne]`` (valid for the first len(links) rows).
    ``autotune`` builds the plan with the autotuner's choice for its shape."""

    def __init__(self, latt_size, Ne, num_nabla, momentum_list, precision="f16x3", batch=None, device=None,
                 evec_dtype=torch.complex128, autotune=False):
        self.device = torch.device(device or "cuda")
        self.latt_size = list(latt_size)
        Lx, Ly, Lz, Lt = latt_size
        self.V3 = Lx * Ly * Lz
        self.Ne = Ne
        if batch is None:
            batch = admit_batch(latt_size, Ne, num_nabla, momentum_list, precision, self.device)
        self.batch = batch
        if autotune:
            from .tune import tuned_plan

            self.plan = tuned_plan(latt_size, Ne, num_nabla, momentum_list, precision, self.device, batch=batch,
                                   evec_dtype=evec_dtype)
        else:
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


@dataclass
class VolumeBinding:
    """One lattice volume of a :class:`MixedVolumeGraph`, bound to caller-owned
    device tensors: ``links`` complex128 ``[3, T, Lz, Ly, Lx, 3, 3]`` (the
    generators' spatial-link layout), ``evecs`` ``[T, Ne, 3*V3]`` c128/c64,
    ``timeslices`` indices into T (repeats allowed), ``out`` complex128
    ``[len(timeslices), Nderiv, Nmom, Ne, Ne]`` (allocated when None)."""

    latt_size: List[int]
    Ne: int
    links: torch.Tensor
    evecs: torch.Tensor
    timeslices: List[int]
    out: torch.Tensor = None


class MixedVolumeGraph:
    """Every timeslice of several lattice volumes (each with its own Ne) in
    ONE captured CUDA graph.

    Each volume gets a batched plan (batch admitted by HBM footprint, the
    volumes' workspaces held at once, largest volume first).  The timeslices
    go in rounds: round r takes the r-th admitted chunk of every volume, builds
    each chunk's chains, contracts all of them with ONE pair-GEMM launch whose
    blocks cover the tiles of every volume (``ed_elemental_gemm_multi``; one
    launch per volume instead when the plans' GEMM forms differ, e.g. a
    factorised momentum list), and combines each chunk into its bound output.
    The graph reads the bound input tensors in place, so a replay (``run()``)
    recomputes everything from their current contents with one host call.
    ``single_launch=False`` keeps one batched pass (and GEMM launch) per
    volume chunk.  ``autotune`` builds each plan with the autotuner's choice
    for its shape (``easydistillation_gb300.tune``)."""

    def __init__(self, volumes: Sequence[VolumeBinding], num_nabla, momentum_list, precision="f16x3",
                 max_batch=8, device=None, autotune=False, reserve=0.1, single_launch=True):
        self.device = torch.device(device or "cuda")
        self.precision = precision
        self.single_launch = single_launch
        self.gemm_launches = None  # GEMM launches per sweep, known after the first run
        self.volumes = list(volumes)
        nd, nm = num_derivative(num_nabla), len(momentum_list)
        self.plans = []
        order = sorted(range(len(self.volumes)), key=lambda i: -self._v3(self.volumes[i]) * self.volumes[i].Ne)
        plans = [None] * len(self.volumes)
        for i in order:
            v = self.volumes[i]
            if v.links.dim() != 7 or v.links.shape[0] != 3 or v.links.dtype != torch.complex128:
                raise ValueError("links must be complex128 [3, T, Lz, Ly, Lx, 3, 3]")
            if v.links.stride(-1) != 1 or v.links.stride(-2) != 3 or v.links.stride(-3) != 9:
                raise ValueError("links must have contiguous 3x3 matrices with unit site stride 9")
            V3 = self._v3(v)
            if v.links.stride(3) != 9 * v.latt_size[0] or v.links.stride(2) != 9 * V3 // v.latt_size[2]:
                raise ValueError("links must be contiguous over the sites of a timeslice")
            if v.out is None:
                v.out = torch.empty((len(v.timeslices), nd, nm, v.Ne, v.Ne), dtype=torch.complex128,
                                    device=self.device)
            n = len(v.timeslices)
            b = min(max_batch, n, admit_batch(v.latt_size, v.Ne, num_nabla, momentum_list, precision, self.device,
                                              max_batch=max_batch, reserve=reserve, static_buffers=False,
                                              forms=(True, "left") if autotune else (True,)))
            if autotune:
                from .tune import factorise_options, tuned_plan

                # one GEMM launch per round takes the volumes on the library's default GEMM form for the momentum
                # list (on chip unless it is close to a product set); the factorisation with every phase on the
                # left (short lists) runs a launch of its own and is measured against it
                forms = None
                if single_launch:
                    forms = [f for f in factorise_options(v.latt_size, v.Ne, num_nabla, momentum_list, precision)
                             if f in (True, "left")]
                plan = tuned_plan(v.latt_size, v.Ne, num_nabla, momentum_list, precision, self.device, batch=b,
                                  evec_dtype=v.evecs.dtype, forms=forms)
            else:
                plan = ElementalPlan(v.latt_size, v.Ne, num_nabla, momentum_list, precision, self.device, batch=b)
            plan.workspace()  # held now, so the next volume's admission sees it
            plans[i] = plan
        self.plans = plans
        self.graph = None

    @staticmethod
    def _v3(v):
        return v.latt_size[0] * v.latt_size[1] * v.latt_size[2]

    def _launch(self):
        if not self.single_launch:
            for v, plan in zip(self.volumes, self.plans):
                ts = list(v.timeslices)
                for s0 in range(0, len(ts), plan.batch):
                    chunk = ts[s0 : s0 + plan.batch]
                    plan.run_batch([v.links[:, t] for t in chunk], v.links.stride(0), 9,
                                   [v.evecs[t] for t in chunk], [v.out[s0 + j] for j in range(len(chunk))])
            self.gemm_launches = self.passes()
            return
        launches = 0
        nround = max(-(-len(v.timeslices) // p.batch) for v, p in zip(self.volumes, self.plans))
        for r in range(nround):
            members = []  # (volume, plan, first output row, timeslices) of this round
            for v, plan in zip(self.volumes, self.plans):
                chunk = list(v.timeslices)[r * plan.batch : (r + 1) * plan.batch]
                if chunk:
                    members.append((v, plan, r * plan.batch, chunk))
            for v, plan, s0, chunk in members:
                plan.run_batch_begin([v.links[:, t] for t in chunk], v.links.stride(0), 9, [v.evecs[t] for t in chunk])
            launches += gemm_multi([m[1] for m in members], [len(m[3]) for m in members])
            for v, plan, s0, chunk in members:
                plan.run_batch_end([v.out[s0 + j] for j in range(len(chunk))])
        self.gemm_launches = launches

    def capture(self):
        self._launch()  # warm-up outside the capture
        torch.cuda.synchronize(self.device)
        self.check_status()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self._launch()
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = g
        return g

    def run(self):
        """Replay the graph (captured on first use); returns the bound outputs."""
        if self.graph is None:
            self.capture()
        self.graph.replay()
        return [v.out for v in self.volumes]

    def passes(self) -> int:
        """Batched passes in the graph."""
        return sum(-(-len(v.timeslices) // p.batch) for v, p in zip(self.volumes, self.plans))

    def check_status(self):
        if self.precision != "fp64":
            for p in self.plans:
                p.check_status()


def run_mixed_volumes(groups: Dict[str, VolumeGroup], links: Dict[str, torch.Tensor],
                      evecs: Dict[str, torch.Tensor], num_nabla, momentum_list, precision="f16x3",
                      max_batch=8, device=None, autotune=False, single_launch=True):
    """Elementals for several lattice volumes (each with its own Ne), all in
    one graphed pass (:class:`MixedVolumeGraph`).  ``links[name]``:
    ``[3, Lt, Lz, Ly, Lx, 3, 3]``; ``evecs[name]``: ``[Lt, Ne, V3*3]``.
    Returns {name: [n_t, Nderiv, Nmom, Ne, Ne]}."""
    names = list(groups)
    vols = [VolumeBinding(groups[n].latt_size, groups[n].Ne, links[n], evecs[n], list(groups[n].timeslices))
            for n in names]
    mv = MixedVolumeGraph(vols, num_nabla, momentum_list, precision, max_batch, device, autotune,
                          single_launch=single_launch)
    outs = mv.run()
    mv.check_status()
    return dict(zip(names, outs))
