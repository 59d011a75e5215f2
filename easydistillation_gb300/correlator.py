"""Meson two-point correlators from elementals and perambulators (GPU, torch).

Mirrors ``lattice/correlator/one_particle.py:12-77`` (``twopoint``) with the
operator data already assembled (``lattice/data.py:7-33``): an operator is a
pair ``(gammas [X, 4, 4], elementals [X, Lt, Ne, Ne])`` of X parts.  The
contraction is the reference's
``"tijab,xjk,xtbc,tklcd,yli,yad->t"`` with ``tau_bw = g5 tau^dag g5`` and the
source gamma ``g4 Gamma^* g4``; it runs as a chain of complex GEMMs on the
device (cuBLAS through torch).  The gamma matrices follow
``lattice/insertion/gamma.py`` (``gamma(n) = g0^(n&1) g1^(n&2) g2^(n&4) g3^(n&8)``).
"""

from __future__ import annotations

from functools import lru_cache
from typing import Iterable, List, Sequence, Tuple

import torch

_G = {
    0: [[0, 0, 0, 1j], [0, 0, 1j, 0], [0, -1j, 0, 0], [-1j, 0, 0, 0]],
    1: [[0, 0, 0, -1], [0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0]],
    2: [[0, 0, 1j, 0], [0, 0, 0, -1j], [-1j, 0, 0, 0], [0, 1j, 0, 0]],
    3: [[0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0], [0, 1, 0, 0]],
}


@lru_cache(maxsize=None)
def _gamma_cpu(n: int) -> torch.Tensor:
    if not (0 <= n <= 15):
        raise ValueError("gamma index must be in 0..15")
    m = torch.eye(4, dtype=torch.complex128)
    for bit in range(4):
        if n & (1 << bit):
            m = m @ torch.tensor(_G[bit], dtype=torch.complex128)
    return m


def gamma(n: int, device=None) -> torch.Tensor:
    """The 4x4 matrix ``gamma(n)`` of the reference's insertion table."""
    return _gamma_cpu(n).to(device or "cpu")


def twopoint_source(tau: torch.Tensor, gammas: torch.Tensor, elementals: torch.Tensor, t_src: int,
                    tau_bw: torch.Tensor = None) -> torch.Tensor:
    """``ret[t]`` for one source timeslice (before the overall minus sign).

    ``tau``: perambulator of this source ``[Lt, 4, 4, Ne, Ne]``; ``gammas``
    ``[X, 4, 4]``; ``elementals`` ``[X, Lt, Ne, Ne]``."""
    dev = tau.device
    g15, g8 = gamma(15, dev), gamma(8, dev)
    if tau_bw is None:
        tau_bw = torch.einsum("ii,tjiba,jj->tijab", g15, tau.conj(), g15)
    gamma_src = torch.einsum("ij,xkj,kl->xil", g8, gammas.conj(), g8)
    phi_t = torch.roll(elementals, -t_src, 1)
    phi_src = elementals[:, t_src].conj()
    # contraction order chosen for GEMM shapes: (tau_bw . Gamma_x . E_x(t)) then (. tau . gsrc_y . E_y(src)^*)
    left = torch.einsum("tijab,xjk,xtbc->tikac", tau_bw, gammas, phi_t)
    right = torch.einsum("tklcd,yli,yad->tkica", tau, gamma_src, phi_src)
    return torch.einsum("tikac,tkica->t", left, right)


def twopoint(operators: Sequence[Tuple[torch.Tensor, torch.Tensor]], perambulator, timeslices: Iterable[int],
             Lt: int, usedNe: int = None, is_sum_over_source_t: bool = True) -> torch.Tensor:
    """``C[op, t]`` like ``lattice/correlator/one_particle.py:12-77``.

    ``operators``: list of ``(gammas [X,4,4], elementals [X, Lt, Ne, Ne])``;
    ``perambulator``: indexable as ``[t_src]`` -> ``[Lt, 4, 4, Ne, Ne]``
    (device tensor or host array)."""
    ts = list(timeslices)
    dev = operators[0][1].device
    ret = torch.zeros((len(operators), len(ts), Lt), dtype=torch.complex128, device=dev)
    for it, t_src in enumerate(ts):
        tau = torch.as_tensor(perambulator[t_src]).to(dev)
        if usedNe is not None:
            tau = tau[..., :usedNe, :usedNe]
        for k, (gm, el) in enumerate(operators):
            e = el if usedNe is None else el[..., :usedNe, :usedNe]
            ret[k, it] = twopoint_source(tau, gm.to(dev), e, t_src)
    return -ret.mean(1) if is_sum_over_source_t else -ret
