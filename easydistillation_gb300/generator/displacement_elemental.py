"""GB300 drop-in for ``lattice.generator.DisplacementElementalGenerator``.

Same constructor, ``load``, ``calc``, ``project_SU3`` and ``stout_smear`` as
``lattice/generator/displacement_elemental.py:11-214``:
``E[dist, p, i, j] = sum_x phase_p(x) conj(V_i(x)) . R^dist_j(x)`` where
``R^0 = V`` and ``R^dist`` is the mean of the six straight-line parallel
transports of ``V`` over ``dist`` links (``_D`` at ``:53-71``; V rounded to
complex64 as at ``:44,88-89``).  The transports run in the library's
one-sided transport kernel, the contraction in its pair-contraction kernels
(``precision`` as for ``ElementalGenerator``; FP64 by default).
"""

from __future__ import annotations

from typing import List, Tuple

import torch

from ..backend import to_backend
from ..insertion import MomentumPhase
from ..ops import PairPlan, links_to_soa, mean_c128, parallel_transport, vectors_to_planes
from .elemental import ElementalGenerator, gauge_to_device

NC = 3


class DisplacementElementalGenerator:
    def __init__(self, latt_size: List[int], gauge_field, eigenvector, distance: int = 0,
                 momentum_list: List[Tuple[int]] = [(0, 0, 0)], *, precision: str = "fp64", device=None) -> None:
        self.device = torch.device(device or "cuda")
        self.latt_size = latt_size
        self.gauge_field = gauge_field
        self.eigenvector = eigenvector
        self.momentum_list = momentum_list
        self.num_momentum = len(momentum_list)
        self.Ne = eigenvector.Ne
        self.distance = distance
        self.precision = precision
        self._U = None
        self._VPV = torch.zeros((distance + 1, self.num_momentum, self.Ne, self.Ne), dtype=torch.complex128,
                                device=self.device)
        self._eigenvector_data = None
        self._momentum_phase = MomentumPhase(latt_size, self.device)
        self._pair = PairPlan(latt_size, self.Ne, distance + 1, momentum_list, 0, 0, distance + 1, precision,
                              self.device)
        self._reader = ElementalGenerator.__new__(ElementalGenerator)  # borrow the eigenvector staging
        self._reader.latt_size, self._reader.Ne, self._reader._stage = latt_size, self.Ne, None
        self._reader.device = self.device

    def load(self, key: str):
        self._U = gauge_to_device(self.gauge_field.load(key), self.latt_size, self.device)
        self._links = links_to_soa(self._U, self.latt_size)
        self._eigenvector_data = self.eigenvector.load(key)

    def project_SU3(self):
        """Iterative projection of the loaded spatial links back onto SU(3)
        (``displacement_elemental.py:98-108``); later ``calc`` calls transport
        with the projected links."""
        from .eigenvector import project_su3_

        self._require_links()
        project_su3_(self._U)
        self._links = links_to_soa(self._U, self.latt_size)

    def stout_smear(self, nstep: int, rho: float):
        """``nstep`` 3D stout steps of weight ``rho`` on the loaded spatial
        links (``displacement_elemental.py:202-214``); later ``calc`` calls
        transport with the smeared links."""
        from .eigenvector import stout_smear_links_

        self._require_links()
        stout_smear_links_(self._U, self.latt_size, nstep, rho)
        self._links = links_to_soa(self._U, self.latt_size)

    def _require_links(self):
        if self._U is None:
            raise RuntimeError("call load(key) before smearing or projecting the links")

    def calc(self, t: int):
        if self._U is None:
            raise RuntimeError("call load(key) before calc(t)")
        Lx, Ly, Lz, Lt = self.latt_size
        V3 = Lx * Ly * Lz
        Ne, D = self.Ne, self.distance
        self._reader._eigenvector_data = self._eigenvector_data
        Vr = self._reader._read_vectors(t).view(Ne, V3, NC)
        V = vectors_to_planes(Vr, V3, torch.complex128, round_c64=True)  # [Ne, 3, V3]
        links = self._links[t]
        chains = torch.empty((D + 1, Ne, NC, V3), dtype=torch.complex128, device=self.device)
        chains[0] = V
        W = torch.empty((6, Ne, NC, V3), dtype=torch.complex128, device=self.device)
        W2 = torch.empty_like(W)
        for dist in range(1, D + 1):
            for d in range(3):
                parallel_transport(links, V if dist == 1 else W[d], self.latt_size, d, +1, out=W2[d])
                parallel_transport(links, V if dist == 1 else W[5 - d], self.latt_size, d, -1, out=W2[5 - d])
            W, W2 = W2, W
            mean_c128(W, out=chains[dist])
        src = chains if self.precision == "fp64" else chains.to(torch.complex64)
        G = self._pair.run(src)  # [Nmom, Ne, (D+1)*Ne]
        self._VPV.copy_(G.view(self.num_momentum, Ne, D + 1, Ne).permute(2, 0, 1, 3))
        return to_backend(self._VPV)
