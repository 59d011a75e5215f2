"""Operator metadata used by the hot path: derivative index scheme, momentum
lists and momentum phases.

Mirrors ``lattice/insertion/derivative.py:23-33`` (``derivative``),
``lattice/insertion/mom_dict.py:5-33,162-175`` (``mom_dict_to_list`` for
|p|^2 <= 1 and <= 3) and ``lattice/insertion/phase.py:6-53``
(``MomentumPhase``), whose tables are computed on the GPU in FP64.
"""

from __future__ import annotations

from typing import List, Sequence, Tuple

import torch

_MOM3 = (
    "0 0 0", "0 0 1", "0 0 -1", "0 1 0", "0 -1 0", "1 0 0", "-1 0 0", "0 1 1", "0 1 -1",
    "0 -1 1", "0 -1 -1", "1 0 1", "1 0 -1", "-1 0 1", "-1 0 -1", "1 1 0", "1 -1 0", "-1 1 0",
    "-1 -1 0", "1 1 1", "1 1 -1", "1 -1 1", "1 -1 -1", "-1 1 1", "-1 1 -1", "-1 -1 1", "-1 -1 -1",
)


def derivative(n: int) -> Tuple[int, ...]:
    """Operator index -> tuple of directions: 0 -> (), 1..3 -> (0,),(1,),(2,),
    4 + 3a + b -> (a, b), and so on in base 3."""
    if n < 0:
        raise ValueError("derivative index must be non-negative")
    length, block = 0, 1
    while n >= block:
        n -= block
        length += 1
        block *= 3
    out = [0] * length
    for k in range(length - 1, -1, -1):
        out[k] = n % 3
        n //= 3
    return tuple(out)


def num_derivative(num_nabla: int) -> int:
    return (3 ** (num_nabla + 1) - 1) // 2


def mom_dict_to_list(mom: int = 3) -> List[Tuple[int, int, int]]:
    if mom == 1:
        return [(0, 0, 0)]
    if mom == 3:
        return [tuple(int(v) for v in s.split(" ")) for s in _MOM3]
    raise ValueError(f"Unknown mom max = {mom}")


class MomentumPhase:
    """Per-site phases ``exp(+2*pi*i*(px*x/Lx + py*y/Ly + pz*z/Lz))`` as FP64
    device tensors ``[Lz, Ly, Lx]``, cached per momentum."""

    def __init__(self, latt_size: Sequence[int], device=None) -> None:
        self.latt_size = list(latt_size)
        self.device = device
        self.cache = {}

    def get(self, np: Sequence[int]) -> torch.Tensor:
        from .ops import momentum_phases

        key = tuple(int(v) for v in np)
        if key not in self.cache:
            self.cache[key] = momentum_phases(self.latt_size, [key], self.device)[0]
        return self.cache[key]
